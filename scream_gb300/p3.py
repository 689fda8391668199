"""Host-side mirror of the EAMxx P3 call surface over libp3x.

``P3Context`` owns the lookup tables (``P3LookupTables`` + ``p3_init``,
components/eamxx/src/physics/p3/p3_f90.cpp:103-113); ``P3Context.p3_main``
is ``Functions<Real,Device>::p3_main`` (p3_functions.hpp:1355-1369) on
device tensors; ``P3Microphysics`` mirrors the atmosphere-process plugin
(components/eamxx/src/physics/p3/eamxx_p3_process_interface.hpp:22-444,
eamxx_p3_run.cpp:5-45) for resident device state.

Device memory and streams come from PyTorch; every computation is a CUDA
kernel of libp3x.  There is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Dict, Optional

import numpy as np

from . import _lib as L

try:  # torch is plumbing for device memory and streams
    import torch
except Exception:  # pragma: no cover - torch is present in every supported environment
    torch = None


def _ptr(t) -> int:
    return 0 if t is None else int(t.data_ptr())


def _stream_handle(stream=None) -> int:
    if torch is None:
        return 0
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def field_shape(name: str, ncol: int, nlev: int):
    if name in L.SURFACE_FIELDS:
        return (ncol,)
    if name in L.INTERFACE_FIELDS:
        return (ncol, nlev + 1)
    return (ncol, nlev)


def generate_inputs(kind: int, seed: int, ncol: int, nlev: int, col0: int = 0) -> Dict[str, np.ndarray]:
    """Synthetic P3 inputs (host float64 arrays of shape (ncol, nlev)).

    kind 0: standard-atmosphere columns with one cloud layer (RH ~ U(0.3, 1.05));
    kind 1: same with RH ~ U(0.9, 1.05) in even columns; kind 2: the reference's
    "mixed" test case.  Columns are generated independently from (seed, column).
    """
    lib = L.load()
    arrs = {n: np.zeros((ncol, nlev), dtype=np.float64) for n in L.INPUT_FIELDS}
    ptrs = (C.c_void_p * len(L.INPUT_FIELDS))(*[a.ctypes.data for a in arrs.values()])
    L.check("p3x_workload_generate",
            lib.p3x_workload_generate(kind, seed, col0, ncol, nlev, ptrs, nlev))
    return arrs


@dataclass
class P3Fields:
    """All arrays of one P3 call (device tensors, level-contiguous)."""
    ncol: int
    nlev: int
    t: Dict[str, "torch.Tensor"] = field(default_factory=dict)

    @classmethod
    def allocate(cls, ncol: int, nlev: int, device="cuda"):
        f = cls(ncol, nlev)
        for n in L.ALL_FIELDS:
            f.t[n] = torch.zeros(field_shape(n, ncol, nlev), dtype=torch.float64, device=device)
        return f

    @classmethod
    def from_inputs(cls, inputs: Dict[str, np.ndarray], device="cuda"):
        ncol, nlev = inputs["qc"].shape
        f = cls.allocate(ncol, nlev, device)
        for n in L.INPUT_FIELDS:
            f.t[n].copy_(torch.from_numpy(np.ascontiguousarray(inputs[n])))
        return f

    def prog(self):
        return L.PrognosticState(*[_ptr(self.t[n]) for n in L.PROG_FIELDS])

    def din(self):
        return L.DiagnosticInputs(*[_ptr(self.t[n]) for n in L.DIAG_IN_FIELDS])

    def dout(self):
        return L.DiagnosticOutputs(*[_ptr(self.t[n]) for n in L.DIAG_OUT_FIELDS])

    def hist(self):
        return L.HistoryOnly(*[_ptr(self.t[n]) for n in L.HIST_FIELDS])

    @classmethod
    def allocate_host(cls, ncol: int, nlev: int, pinned: bool = True):
        """Host (page-locked by default) arrays of one call, for
        :meth:`P3Context.p3_main_host`."""
        f = cls(ncol, nlev)
        for n in L.ALL_FIELDS:
            f.t[n] = torch.zeros(field_shape(n, ncol, nlev), dtype=torch.float64, pin_memory=pinned)
        return f

    def to_host(self) -> Dict[str, np.ndarray]:
        return {n: v.detach().cpu().numpy() for n, v in self.t.items()}

    def desc(self, dt: float, precision: int, predictNc=True, prescribedCCN=True, it=1):
        return L.InstanceDesc(self.prog(), self.din(), self.dout(), self.hist(),
                              L.Layout(self.nlev, self.nlev + 1), self.ncol, self.nlev, dt, it,
                              int(predictNc), int(prescribedCCN), precision)


class P3Context:
    """Lookup tables on the device (generated in-process, or read from the
    official ``p3_lookup_table_1.dat-v4.1.1`` text file)."""

    def __init__(self, table_file: Optional[str] = None):
        self.lib = L.load()
        self.h = C.c_void_p()
        info = C.c_int(0)
        rc = self.lib.p3x_context_create(table_file.encode() if table_file else None,
                                         C.byref(self.h), C.byref(info))
        L.check("p3x_context_create", rc)

    def close(self):
        if self.h:
            self.lib.p3x_context_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tables(self) -> Dict[str, np.ndarray]:
        shp = {"ice": (5, 4, 50, 12), "collect": (5, 4, 50, 30, 2), "vn": (300, 10), "vm": (300, 10),
               "revap": (300, 10), "mu_r": (150,), "dnu": (16,)}
        out = {k: np.zeros(s) for k, s in shp.items()}
        args = [out[k].ctypes.data_as(L._dp) for k in shp]
        L.check("p3x_context_get_tables", self.lib.p3x_context_get_tables(self.h, *args))
        return out

    def set_launch_config(self, precision: int, lanes=None, columns_per_block=None, table_staging=None,
                          blocks_per_sm=None):
        """Launch configuration of a precision form; arguments left at None keep
        their current value (defaults: FP64 16 lanes, FP32-bulk 32, both 4
        columns per CTA, tables through L1)."""
        cur = self.launch_config(precision)
        pick = lambda v, k: cur[k] if v is None else v  # noqa: E731
        cfg = L.LaunchConfig(pick(lanes, "lanes_per_column"), pick(columns_per_block, "columns_per_block"),
                             pick(table_staging, "table_staging"), pick(blocks_per_sm, "blocks_per_sm"))
        L.check("p3x_set_launch_config", self.lib.p3x_set_launch_config(self.h, precision, C.byref(cfg)))

    def launch_config(self, precision: int) -> dict:
        cfg = L.LaunchConfig()
        L.check("p3x_get_launch_config", self.lib.p3x_get_launch_config(self.h, precision, C.byref(cfg)))
        return cfg.as_dict()

    def p3_main(self, f: P3Fields, dt: float, precision: int = L.P3X_FP64, runtime: L.Runtime = None,
                predictNc=True, prescribedCCN=True, it=1, stream=None, sync=True) -> float:
        """One P3 step in place on ``f``; returns the kernel time in microseconds
        (sync) or 0.0 (async; errors then surface in :meth:`check`)."""
        rt = runtime if runtime is not None else L.default_runtime()
        infra = L.Infrastructure(dt, it, 1, f.ncol, 1, f.nlev, int(predictNc), int(prescribedCCN), None)
        prog, din, dout, hist = f.prog(), f.din(), f.dout(), f.hist()
        lay = L.Layout(f.nlev, f.nlev + 1)
        sh = _stream_handle(stream)
        if sync:
            us = C.c_double(0)
            rc = self.lib.p3x_main(self.h, C.byref(rt), C.byref(prog), C.byref(din), C.byref(dout),
                                   C.byref(infra), C.byref(hist), f.ncol, f.nlev, C.byref(lay),
                                   precision, sh, C.byref(us))
            L.check("p3x_main", rc)
            return us.value
        rc = self.lib.p3x_main_async(self.h, C.byref(rt), C.byref(prog), C.byref(din), C.byref(dout),
                                     C.byref(infra), C.byref(hist), f.ncol, f.nlev, C.byref(lay),
                                     precision, sh)
        L.check("p3x_main_async", rc)
        return 0.0

    def handover_bytes(self, ncol: int, nlev: int) -> int:
        n = C.c_int64(0)
        L.check("p3x_handover_bytes", self.lib.p3x_handover_bytes(int(ncol), int(nlev), C.byref(n)))
        return n.value

    def allocate_handover(self, ncol: int, nlev: int, device="cuda"):
        """A zeroed device buffer for :meth:`p3_main_stages` (uint8 tensor)."""
        return torch.zeros(self.handover_bytes(ncol, nlev), dtype=torch.uint8, device=device)

    @staticmethod
    def handover_views(buf, ncol: int, nlev: int):
        """(rows, cflag) views of a hand-over buffer: rows (5, ncol, nlev)
        float64 (temperature after part1, density, rhofacr, rhofaci, acn),
        cflag (ncol,) int32."""
        nd = 5 * ncol * nlev
        rows = buf[: nd * 8].view(torch.float64).view(5, ncol, nlev)
        cflag = buf[nd * 8: nd * 8 + ncol * 4].view(torch.int32)
        return rows, cflag

    def p3_main_stages(self, f: P3Fields, dt: float, stages: int, handover, precision: int = L.P3X_FP64,
                       runtime: L.Runtime = None, predictNc=True, prescribedCCN=True, it=1, stream=None):
        """Runs the subset ``stages`` (P3X_STAGE_* bits) of the step's three
        kernels on ``f`` with the hand-over in ``handover`` (p3x_main_stages),
        then synchronises and checks the device status."""
        rt = runtime if runtime is not None else L.default_runtime()
        infra = L.Infrastructure(dt, it, 1, f.ncol, 1, f.nlev, int(predictNc), int(prescribedCCN), None)
        rc = self.lib.p3x_main_stages(self.h, C.byref(rt), C.byref(f.prog()), C.byref(f.din()),
                                      C.byref(f.dout()), C.byref(infra), C.byref(f.hist()), f.ncol, f.nlev,
                                      C.byref(L.Layout(f.nlev, f.nlev + 1)), precision, int(stages),
                                      _ptr(handover), _stream_handle(stream))
        L.check("p3x_main_stages", rc)
        self.check(stream)

    def p3_main_host(self, f: P3Fields, dt: float, precision: int = L.P3X_FP64, runtime: L.Runtime = None,
                     predictNc=True, prescribedCCN=True, it=1, chunk_cols=0) -> float:
        """One P3 step on HOST arrays (``P3Fields.allocate_host``), copies
        overlapped with the kernels chunk by chunk (p3x_main_host); returns
        the time from first upload to last download in microseconds."""
        rt = runtime if runtime is not None else L.default_runtime()
        infra = L.Infrastructure(dt, it, 1, f.ncol, 1, f.nlev, int(predictNc), int(prescribedCCN), None)
        us = C.c_double(0)
        rc = self.lib.p3x_main_host(self.h, C.byref(rt), C.byref(f.prog()), C.byref(f.din()), C.byref(f.dout()),
                                    C.byref(infra), C.byref(f.hist()), f.ncol, f.nlev,
                                    C.byref(L.Layout(f.nlev, f.nlev + 1)), precision, chunk_cols, C.byref(us))
        L.check("p3x_main_host", rc)
        return us.value

    def _interface(self, host_fields: Dict[str, "torch.Tensor"]):
        return L.InterfaceFields(*[(_ptr(host_fields[n]) if host_fields.get(n) is not None else None)
                                   for n in L.HOST_MODEL_FIELDS])

    def preamble(self, host_fields: Dict[str, "torch.Tensor"], f: P3Fields, stream=None):
        """P3Microphysics preamble on the device: host-model fields (pmid,
        pseudo_density(_dry), cld_frac_t, T_atm) and wet mixing ratios in ``f``
        -> P3 inputs in ``f`` (dry mixing ratios, th, inv_exner, dz, cloud
        fractions, dry qv_prev)."""
        itf = self._interface(host_fields)
        L.check("p3x_preamble", self.lib.p3x_preamble(C.byref(itf), C.byref(f.prog()), C.byref(f.din()), f.ncol,
                                                      f.nlev, C.byref(L.Layout(f.nlev, f.nlev + 1)),
                                                      _stream_handle(stream)))

    def postamble(self, host_fields: Dict[str, "torch.Tensor"], f: P3Fields, dt: float, stream=None):
        """P3Microphysics postamble on the device (T_atm, T_prev, wet mixing
        ratios, qv_prev, effective radii in microns, precipitation mass,
        boundary fluxes)."""
        itf = self._interface(host_fields)
        L.check("p3x_postamble", self.lib.p3x_postamble(C.byref(itf), C.byref(f.prog()), C.byref(f.din()),
                                                        C.byref(f.dout()), f.ncol, f.nlev,
                                                        C.byref(L.Layout(f.nlev, f.nlev + 1)), float(dt),
                                                        _stream_handle(stream)))

    def _eam(self, eam: Dict[str, "torch.Tensor"], subgrid: bool, method: int):
        def p(n):
            t = eam.get(n)
            return _ptr(t) if t is not None else None
        e = L.EamFields()
        for n in L.EAM_STATE + L.EAM_PBUF_IN + ["t_prev", "qv_prev", "ptend_s"] + L.EAM_DIAG:
            setattr(e, n, p(n))
        for i, s in enumerate(L.EAM_SPECIES):
            e.q[i] = p(s)
            e.ptend_q[i] = p("ptend_" + s)
        e.subgrid_clouds = 1 if subgrid else 0
        e.precip_frac_method = int(method)
        return e

    def eam_tend_pre(self, eam: Dict[str, "torch.Tensor"], f: P3Fields, subgrid: bool = True,
                     method: int = L.PRECIP_FRAC_MAX_OVERLAP, stream=None):
        """EAM driver preparation (micro_p3_tend): P3 inputs in ``f`` from the
        EAM state in ``eam`` (device tensors named as in p3x_eam_fields; the
        nine constituents by their driver names, interfaces (ncol, nlev+1))."""
        e = self._eam(eam, subgrid, method)
        L.check("p3x_eam_tend_pre", self.lib.p3x_eam_tend_pre(C.byref(e), C.byref(f.prog()), C.byref(f.din()),
                                                              f.ncol, f.nlev, C.byref(L.Layout(f.nlev, f.nlev + 1)),
                                                              _stream_handle(stream)))

    def eam_tend_post(self, eam: Dict[str, "torch.Tensor"], f: P3Fields, dt: float, stream=None):
        """EAM driver use of the P3 results in ``f``: tendencies, t_prev and
        qv_prev, diagnostics into ``eam`` (optional ones when present)."""
        e = self._eam(eam, True, L.PRECIP_FRAC_MAX_OVERLAP)
        L.check("p3x_eam_tend_post", self.lib.p3x_eam_tend_post(C.byref(e), C.byref(f.prog()), C.byref(f.din()),
                                                                C.byref(f.dout()), C.byref(f.hist()), f.ncol,
                                                                f.nlev, C.byref(L.Layout(f.nlev, f.nlev + 1)),
                                                                float(dt), _stream_handle(stream)))

    def eam_micro_p3_tend(self, eam: Dict[str, "torch.Tensor"], f: P3Fields, dt: float, it: int = 1,
                          precision: int = L.P3X_FP64, predictNc: bool = True, prescribedCCN: bool = False,
                          subgrid: bool = True, method: int = L.PRECIP_FRAC_MAX_OVERLAP, runtime=None,
                          stream=None):
        """micro_p3_tend on the device: preparation, the P3 step and the use of
        its results, asynchronously on ``stream`` (``f``: the working arrays)."""
        e = self._eam(eam, subgrid, method)
        rt = runtime if runtime is not None else L.default_runtime()
        infra = L.Infrastructure(float(dt), int(it), 1, f.ncol, 1, f.nlev, int(predictNc), int(prescribedCCN), None)
        L.check("p3x_eam_micro_p3_tend",
                self.lib.p3x_eam_micro_p3_tend(self.h, C.byref(rt), C.byref(e), C.byref(f.prog()),
                                               C.byref(f.din()), C.byref(f.dout()), C.byref(infra),
                                               C.byref(f.hist()), f.ncol, f.nlev,
                                               C.byref(L.Layout(f.nlev, f.nlev + 1)), int(precision),
                                               _stream_handle(stream)))

    def _cons(self, fields: Dict[str, "torch.Tensor"]):
        return L.ConservationFields(*[(_ptr(fields[n]) if fields.get(n) is not None else None)
                                      for n in L.CONS_FIELDS])

    def column_mass_energy(self, fields: Dict[str, "torch.Tensor"], stream=None):
        """Column mass and energy of host-model fields (the conservation
        check's totals before a process); device tensors of shape (ncol,)."""
        ncol, nlev = fields["qv"].shape
        m = torch.zeros(ncol, dtype=torch.float64, device=fields["qv"].device)
        e = torch.zeros_like(m)
        cf = self._cons(fields)
        L.check("p3x_column_mass_energy", self.lib.p3x_column_mass_energy(
            C.byref(cf), ncol, nlev, nlev, _ptr(m), _ptr(e), _stream_handle(stream)))
        return m, e

    def conservation_check(self, fields: Dict[str, "torch.Tensor"], mass_before, energy_before, dt: float,
                           mass_tol: float = 1e-10, energy_tol: float = 1e-14, stream=None):
        """Mass and energy conservation check after a process: (report dict,
        per-column relative mass errors, per-column relative energy errors).
        Default tolerances are the reference driver's."""
        ncol, nlev = fields["qv"].shape
        me = torch.zeros(ncol, dtype=torch.float64, device=fields["qv"].device)
        ee = torch.zeros_like(me)
        rep = L.ConservationReport()
        cf = self._cons(fields)
        L.check("p3x_conservation_check", self.lib.p3x_conservation_check(
            self.h, C.byref(cf), _ptr(mass_before), _ptr(energy_before), ncol, nlev, nlev, float(dt),
            float(mass_tol), float(energy_tol), _ptr(me), _ptr(ee), C.byref(rep), _stream_handle(stream)))
        return rep.as_dict(), me, ee

    def set_kernel_timing(self, on: bool = True):
        L.check("p3x_set_kernel_timing", self.lib.p3x_set_kernel_timing(self.h, int(bool(on))))

    def kernel_times(self):
        """(part1+part2, sedimentation, part3) durations in ms of the latest
        timed step."""
        ms = (C.c_float * 3)()
        L.check("p3x_kernel_times", self.lib.p3x_kernel_times(self.h, ms))
        return [float(x) for x in ms]

    def set_check_values(self, mode: int):
        """check_values after part3: L.P3X_CHECK_OFF / _RECORD / _FAIL."""
        L.check("p3x_set_check_values", self.lib.p3x_set_check_values(self.h, int(mode)))

    def check_values_report(self, stream=None) -> dict:
        """Out-of-range counts and first locations since the last report (cleared)."""
        rep = L.CheckReport()
        L.check("p3x_check_values_report",
                self.lib.p3x_check_values_report(self.h, _stream_handle(stream), C.byref(rep)))
        return rep.as_dict()

    def check(self, stream=None):
        L.check("p3x_context_check", self.lib.p3x_context_check(self.h, _stream_handle(stream)))

    def budgets(self, f: P3Fields, stream=None):
        """Column total water and energy (FP64, device tensors of shape (ncol,))."""
        w = torch.zeros(f.ncol, dtype=torch.float64, device=f.t["qc"].device)
        e = torch.zeros_like(w)
        prog = f.prog()
        rc = self.lib.p3x_column_budgets(C.byref(prog), _ptr(f.t["dpres"]), _ptr(f.t["inv_exner"]),
                                         f.ncol, f.nlev, f.nlev, _ptr(w), _ptr(e), _stream_handle(stream))
        L.check("p3x_column_budgets", rc)
        return w, e


class P3Batch:
    """Many instances advanced by one persistent launch (optionally a CUDA graph)."""

    def __init__(self, ctx: P3Context, fields, dts, precision: int, runtime: L.Runtime = None,
                 predictNc=True, prescribedCCN=True):
        self.ctx = ctx
        self.fields = list(fields)
        rt = runtime if runtime is not None else L.default_runtime()
        descs = (L.InstanceDesc * len(self.fields))(
            *[f.desc(dt, precision, predictNc, prescribedCCN) for f, dt in zip(self.fields, dts)])
        self.h = C.c_void_p()
        L.check("p3x_batch_create", ctx.lib.p3x_batch_create(ctx.h, C.byref(rt), descs, len(self.fields),
                                                             C.byref(self.h)))
        # a new batch starts from the context's configuration for its precision
        self._cfg = ctx.launch_config(precision)

    def run(self, stream=None):
        L.check("p3x_batch_run", self.ctx.lib.p3x_batch_run(self.h, _stream_handle(stream)))

    def capture_graph(self, stream):
        L.check("p3x_batch_capture_graph", self.ctx.lib.p3x_batch_capture_graph(self.h, _stream_handle(stream)))

    def set_launch_config(self, lanes=None, columns_per_block=None, table_staging=None, blocks_per_sm=None):
        """Launch configuration of the batch; arguments left at None keep their
        current value (initially the context's configuration for the batch's
        precision)."""
        cur = self._cfg
        pick = lambda v, k: cur[k] if v is None else v  # noqa: E731
        cfg = L.LaunchConfig(pick(lanes, "lanes_per_column"), pick(columns_per_block, "columns_per_block"),
                             pick(table_staging, "table_staging"), pick(blocks_per_sm, "blocks_per_sm"))
        L.check("p3x_batch_set_launch_config", self.ctx.lib.p3x_batch_set_launch_config(self.h, C.byref(cfg)))
        self._cfg = cfg.as_dict()

    def autotune(self, reps=3, stream=None):
        cfg = L.LaunchConfig()
        ms = C.c_double(0)
        L.check("p3x_autotune_batch", self.ctx.lib.p3x_autotune_batch(self.h, _stream_handle(stream), reps,
                                                                      C.byref(cfg), C.byref(ms)))
        self._cfg = cfg.as_dict()
        return cfg.as_dict(), ms.value

    def close(self):
        if self.h:
            self.ctx.lib.p3x_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class P3Server:
    """Continuous-batching request loop over resident P3 instances
    (p3x_server_* in include/p3x.h): admission under a device-memory budget,
    up to ``max_inflight`` overlapping dispatches, p50/p99 latency."""

    def __init__(self, ctx: P3Context, budget_bytes: int = 120 * 10**9, max_inflight: int = 4,
                 runtime: L.Runtime = None):
        self.ctx = ctx
        rt = runtime if runtime is not None else L.default_runtime()
        self.h = C.c_void_p()
        L.check("p3x_server_create", ctx.lib.p3x_server_create(ctx.h, C.byref(rt), int(budget_bytes),
                                                               int(max_inflight), C.byref(self.h)))

    def submit(self, instance_id: int, ncol: int, nlev: int, precision: int, total_steps: int = 1,
               seed: int = 0, dt: float = 300.0, arrival_s: float = 0.0):
        L.check("p3x_server_submit", self.ctx.lib.p3x_server_submit(
            self.h, int(instance_id), int(ncol), int(nlev), int(precision), int(total_steps), int(seed),
            float(dt), float(arrival_s)))

    def drain(self) -> dict:
        st = L.ServeStats()
        L.check("p3x_server_drain", self.ctx.lib.p3x_server_drain(self.h, C.byref(st)))
        return st.as_dict()

    def run_poisson(self, rate_hz: float, n_sessions: int, max_ncol: int = 65536, seed: int = 4) -> dict:
        st = L.ServeStats()
        L.check("p3x_server_run_poisson", self.ctx.lib.p3x_server_run_poisson(
            self.h, float(rate_hz), int(n_sessions), int(max_ncol), int(seed), C.byref(st)))
        return st.as_dict()

    def set_latency_policy(self, on: bool = True, large_grid_share: float = 0.875):
        """Dispatch policy (p3x_server_set_latency_policy): on favours small
        requests' latency, off packs every ready request for throughput."""
        L.check("p3x_server_set_latency_policy", self.ctx.lib.p3x_server_set_latency_policy(
            self.h, int(bool(on)), float(large_grid_share)))

    def set_sm_partition(self, small_sms: int, small_max_cl: int = 1 << 15):
        """SM partition (p3x_server_set_sm_partition): the last slot on its own
        green context of at least ``small_sms`` SMs, taking only instances of
        at most ``small_max_cl`` column-levels; 0 removes it.  Returns the SM
        counts (small, rest)."""
        sms = (C.c_int32 * 2)()
        L.check("p3x_server_set_sm_partition", self.ctx.lib.p3x_server_set_sm_partition(
            self.h, int(small_sms), int(small_max_cl), sms))
        return int(sms[0]), int(sms[1])

    def set_dispatch_chunk(self, max_cl: int):
        """Dispatch chunking (p3x_server_set_dispatch_chunk): dispatches above
        ``max_cl`` column-levels run as consecutive launches of at most that
        size (default 2**18); 0 launches each dispatch at once."""
        L.check("p3x_server_set_dispatch_chunk", self.ctx.lib.p3x_server_set_dispatch_chunk(self.h, int(max_cl)))

    def calibrate(self):
        """Isolated service times (p3x_server_calibrate); later stats report slowdowns."""
        L.check("p3x_server_calibrate", self.ctx.lib.p3x_server_calibrate(self.h))

    def isolated_ms(self, precision: int, nlev: int, ncol: int) -> float:
        ms = C.c_double(0)
        L.check("p3x_server_isolated_ms", self.ctx.lib.p3x_server_isolated_ms(
            self.h, int(precision), int(nlev), int(ncol), C.byref(ms)))
        return ms.value

    def export_instance(self, instance_id: int, ncol: int, nlev: int) -> np.ndarray:
        """The instance's 23 input fields, (23, ncol, nlev) float64 (checkpoint)."""
        out = np.empty((len(L.INPUT_FIELDS), ncol, nlev), dtype=np.float64)
        L.check("p3x_server_export_instance", self.ctx.lib.p3x_server_export_instance(
            self.h, int(instance_id), out.ctypes.data_as(C.POINTER(C.c_double)), int(out.size)))
        return out

    def import_instance(self, instance_id: int, state: np.ndarray, precision: int, dt: float = 300.0):
        """Makes an instance resident from an exported state (resume)."""
        st = np.ascontiguousarray(state, dtype=np.float64)
        _, ncol, nlev = st.shape
        L.check("p3x_server_import_instance", self.ctx.lib.p3x_server_import_instance(
            self.h, int(instance_id), int(ncol), int(nlev), int(precision), float(dt),
            st.ctypes.data_as(C.POINTER(C.c_double)), int(st.size)))

    def read_field(self, instance_id: int, field: int, n: int) -> np.ndarray:
        out = np.empty(n, dtype=np.float64)
        L.check("p3x_server_read_field", self.ctx.lib.p3x_server_read_field(
            self.h, int(instance_id), int(field), out.ctypes.data_as(C.POINTER(C.c_double)), int(n)))
        return out

    def close(self):
        if self.h:
            self.ctx.lib.p3x_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class P3Microphysics:
    """Mirror of the ``P3Microphysics`` atmosphere process for resident device
    state: ``set_grids`` fixes (ncol, nlev), ``initialize`` creates the tables
    and the fields, ``run(dt)`` advances the step counter and calls p3_main
    (eamxx_p3_run.cpp:5-45), ``finalize`` releases everything."""

    def __init__(self, params: Optional[dict] = None):
        params = dict(params or {})
        self.runtime = L.default_runtime()
        for k in L.RUNTIME_FIELDS:
            if k in params:
                setattr(self.runtime, k, float(params[k]))
        if "do_ice_production" in params:
            self.runtime.do_ice_production = int(bool(params["do_ice_production"]))
        self.predictNc = bool(params.get("do_predict_nc", True))
        self.prescribedCCN = bool(params.get("do_prescribed_CCN", True))
        self.precision = int(params.get("precision", L.P3X_FP64))
        self.table_file = params.get("table_file")
        self.ncol = self.nlev = None
        self.ctx = None
        self.fields = None
        self.it = 0

    def type(self):
        return "Physics"

    def name(self):
        return "p3"

    def set_grids(self, ncol: int, nlev: int):
        self.ncol, self.nlev = int(ncol), int(nlev)

    def initialize(self, inputs: Optional[Dict[str, np.ndarray]] = None):
        self.ctx = P3Context(self.table_file)
        if inputs is None:
            self.fields = P3Fields.allocate(self.ncol, self.nlev)
        else:
            self.fields = P3Fields.from_inputs(inputs)
        self.it = 0

    def run(self, dt: float, stream=None) -> float:
        self.it += 1
        return self.ctx.p3_main(self.fields, dt, self.precision, self.runtime, self.predictNc,
                                self.prescribedCCN, self.it, stream)

    def run_process(self, host_fields, dt: float, stream=None) -> float:
        """One atmosphere-process step as run_impl does it
        (eamxx_p3_run.cpp:5-45): preamble (wet -> dry, th, dz, cloud
        fractions), p3_main, postamble (T_atm, T_prev, dry -> wet, qv_prev,
        radii, precipitation mass, boundary fluxes).  ``host_fields`` holds the
        host model's device tensors named as in p3x_interface_fields."""
        self.ctx.preamble(host_fields, self.fields, stream)
        us = self.run(dt, stream)
        self.ctx.postamble(host_fields, self.fields, dt, stream)
        return us

    def finalize(self):
        if self.ctx is not None:
            self.ctx.close()
        self.ctx = None
        self.fields = None
