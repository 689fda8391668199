import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Builds libp3x.so and the oracle once per session (no GPU needed)."""
    from scream_gb300 import build as b
    from oracle import build as ob
    b.build()
    ob.build()
    import scream_gb300
    return scream_gb300.load()


@pytest.fixture(scope="session")
def tables(built):
    from scream_gb300 import _lib as L
    return L.host_tables()


@pytest.fixture(scope="session")
def gpu_ctx(built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import scream_gb300 as p3
    ctx = p3.P3Context()
    yield ctx
    ctx.close()


def oracle_state(inputs):
    """Copies generator inputs into a full oracle state dict (outputs zeroed)."""
    from oracle import p3_oracle as O
    st = {k: np.array(v, dtype=np.float64, copy=True) for k, v in inputs.items()}
    st.update(O.empty_outputs(*inputs["qc"].shape))
    return st


def rel_l2(a, b):
    den = np.linalg.norm(b)
    num = np.linalg.norm(np.asarray(a) - np.asarray(b))
    return num / den if den > 0 else num


def column_water(st):
    g = 9.80616
    return ((st["qv"] + st["qc"] + st["qr"] + st["qi"]) * st["dpres"] / g).sum(axis=1)
