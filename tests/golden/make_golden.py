"""Generates the committed fixtures of tests/golden/.

reference_kats.json
    Known-answer inputs of the reference's conservation-limiter unit tests,
    transcribed from components/eamxx/src/physics/p3/tests/p3_unit_tests.cpp
    (:31 CloudWaterConservationData, :84 RainWaterConservationData,
    :137 IceWaterConservationData); the expected values are the closed-form
    ratios those tests REQUIRE.
mixed_ic_oracle.npz
    Oracle state after 6 steps (dt = 300 s) of the reference's "mixed" initial
    condition (3 columns x 72 levels), for (predict_nc, prescribed_CCN) in
    {(1,1), (0,0), (1,0)} -- the p3_run_and_cmp cases.  A regression pin of
    the oracle across machines (not a reference output: the reference cannot
    be built here).
table_summary.json
    Checksums and sample entries of the generated lookup tables.

Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))


def main():
    from scream_gb300 import _lib as L
    from scream_gb300.p3 import generate_inputs
    from oracle import p3_oracle as O

    kats = {
        "source": "components/eamxx/src/physics/p3/tests/p3_unit_tests.cpp:27-175",
        "cloud_water_conservation": {"qc": 1e-5, "dt": 1.1,
                                     "tend_in": [1e-4, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, 1.0],
                                     "order": ["qc2qr_autoconv", "qc2qr_accret", "qc2qi_collect",
                                               "qc2qi_hetero_freeze", "qc2qr_ice_shed", "qc2qi_berg",
                                               "qi2qv_sublim", "qv2qi_vapdep"]},
        "rain_water_conservation": {"qr": 1e-5, "dt": 1.1,
                                    "tend_in": [0.0, 0.0, 0.0, 0.0, 1e-4, 0.0, 0.0],
                                    "order": ["qc2qr_autoconv", "qc2qr_accret", "qi2qr_melt",
                                              "qc2qr_ice_shed", "qr2qv_evap", "qr2qi_collect",
                                              "qr2qi_immers_freeze"]},
        "ice_water_conservation": {"qi": 1e-5, "dt": 1.1,
                                   "tend_in": [0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1e-4, 0.0],
                                   "order": ["qv2qi_vapdep", "qv2qi_nucleat", "qc2qi_berg", "qr2qi_collect",
                                             "qc2qi_collect", "qr2qi_immers_freeze", "qc2qi_hetero_freeze",
                                             "qi2qv_sublim", "qi2qr_melt"]},
    }
    (HERE / "reference_kats.json").write_text(json.dumps(kats, indent=1) + "\n")

    tables = L.host_tables()
    out = {}
    for pn, pc in [(1, 1), (0, 0), (1, 0)]:
        inp = generate_inputs(2, 0, 3, 72)
        st = {k: np.array(v, copy=True) for k, v in inp.items()}
        st.update(O.empty_outputs(3, 72))
        for it in range(1, 7):
            err, _ = O.p3_main(st, tables, 300.0, predictNc=bool(pn), prescribedCCN=bool(pc), it=it)
            assert err == 0
        for n, v in st.items():
            if n in O.FIELDS_DIN:
                continue
            out[f"p{pn}{pc}_{n}"] = v
    np.savez_compressed(HERE / "mixed_ic_oracle.npz", **out)

    summ = {k: {"sum": float(np.sum(v)), "abs_sum": float(np.sum(np.abs(v))),
                "first": float(v.ravel()[0]), "mid": float(v.ravel()[v.size // 2]),
                "last": float(v.ravel()[-1])} for k, v in tables.items()}
    (HERE / "table_summary.json").write_text(json.dumps(summ, indent=1) + "\n")
    print("wrote", sorted(p.name for p in HERE.iterdir()))


if __name__ == "__main__":
    main()
