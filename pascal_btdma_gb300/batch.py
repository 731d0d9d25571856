"""Uneven batches (include/pbt_batch.h): many systems of different length N
and block size m (1..10) solved by one persistent kernel launch per block size, plus the autotuner
that picks the segmentation and CTA shape per (m, N, nsys) bucket, and CUDA
graph capture of repeated sweeps.

    plan = BatchPlan(m_per_sys, n_per_sys, precision="fp64", tuning=autotune(...))
    pa, pb, pc, pd = plan.pack(ua, ub, uc, ud)      # per-system -> packed (device tensors)
    plan.solve(pa, pb, pc, pd)                      # one persistent launch per block size
    ud = plan.unpack(pd)                            # packed -> per-system

Per-system (caller) layout: system s is the reference layout of one system at
its own offset, A_s[row + N_s*(i + m_s*j)] at mat_off[s], D_s[row + N_s*i] at
vec_off[s] (``plan.user_offsets()``).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
from pathlib import Path

import numpy as np

from . import _native as N
from . import _raise

PBT_BATCH_MAX_BLOCK = 10


class BatchTuning(C.Structure):
    _fields_ = [("seg_len", C.c_int * (N.PBT_MAX_BLOCK + 1)), ("warps_per_cta", C.c_int), ("reserved", C.c_int * 8)]

    @classmethod
    def make(cls, seg_len: dict | None = None, warps_per_cta: int = 4) -> "BatchTuning":
        t = cls()
        N.lib().pbt_batch_tuning_init(C.byref(t))
        for m, v in (seg_len or {}).items():
            t.seg_len[int(m)] = int(v)
        t.warps_per_cta = int(warps_per_cta)
        return t

    def as_dict(self) -> dict:
        return {"seg_len": {m: self.seg_len[m] for m in range(1, N.PBT_MAX_BLOCK + 1)},
                "warps_per_cta": self.warps_per_cta}


_P = C.c_void_p
_LL = C.POINTER(C.c_longlong)
BATCH_SIGNATURES = {
    "pbt_batch_tuning_init": (None, [C.POINTER(BatchTuning)]),
    "pbt_batch_create": (C.c_int, [C.POINTER(_P), C.c_int, _P, _P, C.c_int, C.POINTER(BatchTuning)]),
    "pbt_batch_destroy": (C.c_int, [_P]),
    "pbt_batch_sizes": (C.c_int, [_P, _LL, _LL, _LL, _LL]),
    "pbt_batch_user_offsets": (C.c_int, [_P, _P, _P]),
    "pbt_batch_pack": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "pbt_batch_unpack": (C.c_int, [_P, _P, _P, _P]),
    "pbt_batch_solve": (C.c_int, [_P, _P, _P, _P, _P, _P]),
    "pbt_batch_status": (C.c_int, [_P, _LL, C.POINTER(C.c_int)]),
    "pbt_batch_info": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                 C.POINTER(C.c_int)]),
}
_bound = False


def _lib():
    global _bound
    lib = N.lib()
    if not _bound:
        for name, (res, args) in BATCH_SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _bound = True
    return lib


def _dptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


class BatchPlan:
    def __init__(self, m_per_sys, n_per_sys, precision: str = "fp64", tuning: BatchTuning | dict | None = None):
        import torch  # noqa: F401

        from . import PRECISIONS

        self.m = np.ascontiguousarray(m_per_sys, dtype=np.int32)
        self.n = np.ascontiguousarray(n_per_sys, dtype=np.int32)
        if self.m.shape != self.n.shape or self.m.ndim != 1:
            raise ValueError("m_per_sys and n_per_sys must be 1-D of equal length")
        if isinstance(tuning, dict):
            tuning = BatchTuning.make(tuning.get("seg_len"), tuning.get("warps_per_cta", 4))
        self.tuning = tuning
        self.precision = precision
        h = _P()
        code = _lib().pbt_batch_create(C.byref(h), int(self.m.size), self.m.ctypes.data, self.n.ctypes.data,
                                       PRECISIONS[precision], C.byref(tuning) if tuning is not None else None)
        _raise(code, "BatchPlan")
        self._h = h

    @property
    def nsys(self) -> int:
        return int(self.m.size)

    def sizes(self) -> tuple[int, int, int, int]:
        v = [C.c_longlong() for _ in range(4)]
        _raise(_lib().pbt_batch_sizes(self._h, *(C.byref(x) for x in v)), "BatchPlan.sizes")
        return tuple(int(x.value) for x in v)

    def user_offsets(self) -> tuple[np.ndarray, np.ndarray]:
        mo = np.empty(self.nsys, dtype=np.int64)
        vo = np.empty(self.nsys, dtype=np.int64)
        _raise(_lib().pbt_batch_user_offsets(self._h, mo.ctypes.data, vo.ctypes.data), "BatchPlan.user_offsets")
        return mo, vo

    def info(self) -> dict:
        v = [C.c_int() for _ in range(4)]
        _raise(_lib().pbt_batch_info(self._h, *(C.byref(x) for x in v)), "BatchPlan.info")
        return dict(zip(("tiles", "stage1_items", "stage3_items", "grid_ctas"), (x.value for x in v)))

    def _stream(self, stream):
        import torch

        return C.c_void_p(torch.cuda.current_stream().cuda_stream if stream is None else stream.cuda_stream)

    def pack(self, ua, ub, uc, ud, out=None, stream=None):
        import torch

        _, _, pm, pv = self.sizes()
        if out is None:
            out = tuple(torch.empty(n, dtype=torch.float64, device=ua.device) for n in (pm, pm, pm, pv))
        code = _lib().pbt_batch_pack(self._h, *(_dptr(t) for t in (ua, ub, uc, ud)), *(_dptr(t) for t in out),
                                     self._stream(stream))
        _raise(code, "BatchPlan.pack")
        return out

    def unpack(self, pd, ud=None, stream=None):
        import torch

        _, uv, _, _ = self.sizes()
        if ud is None:
            ud = torch.empty(uv, dtype=torch.float64, device=pd.device)
        _raise(_lib().pbt_batch_unpack(self._h, _dptr(pd), _dptr(ud), self._stream(stream)), "BatchPlan.unpack")
        return ud

    def solve(self, pa, pb, pc, pd, stream=None) -> None:
        code = _lib().pbt_batch_solve(self._h, *(_dptr(t) for t in (pa, pb, pc, pd)), self._stream(stream))
        _raise(code, "BatchPlan.solve")

    def status(self) -> tuple[int, int]:
        ns, to = C.c_longlong(0), C.c_int(0)
        code = _lib().pbt_batch_status(self._h, C.byref(ns), C.byref(to))
        if code not in (N.PBT_OK, N.PBT_ESINGULAR) or to.value:
            _raise(code if code else N.PBT_ECUDA, "BatchPlan.status")
        return int(ns.value), int(to.value)

    def destroy(self) -> None:
        if getattr(self, "_h", None):
            _raise(_lib().pbt_batch_destroy(self._h), "BatchPlan.destroy")
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Autotuner.
# ---------------------------------------------------------------------------
SEG_CANDIDATES = (0, 1024, 512, 256, 128, 64, 32)   # 0: one segment per line
WARP_CANDIDATES = (4, 2)


def bucket_key(m_per_sys, n_per_sys, precision: str) -> str:
    """(m, N, nsys) bucket of a batch: the count of systems per (m, log2 N)
    bin, rounded to 2 significant digits, and nsys to a power of two."""
    m = np.asarray(m_per_sys)
    n = np.asarray(n_per_sys)
    hist = {}
    for mm in np.unique(m):
        sel = n[m == mm]
        b = np.bincount(np.floor(np.log2(sel)).astype(int), minlength=16)
        hist[int(mm)] = [int(float(f"{x:.2g}")) for x in b]
    desc = {"precision": precision, "nsys_log2": int(np.round(np.log2(m.size))), "hist": hist}
    return hashlib.sha1(json.dumps(desc, sort_keys=True).encode()).hexdigest()[:16]


def default_cache() -> Path:
    return Path(os.environ.get("PBT_TUNE_CACHE", str(Path.home() / ".cache" / "pascal_btdma_gb300" / "batch_tuning.json")))


def time_solve(plan: BatchPlan, packed, d0, reps: int = 3) -> float:
    """Median time of one solve (restoring D from d0 before each), seconds."""
    import torch

    pa, pb, pc, pd = packed
    times = []
    for r in range(reps + 1):
        pd.copy_(d0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        plan.solve(pa, pb, pc, pd)
        e1.record()
        torch.cuda.synchronize()
        if r:
            times.append(e0.elapsed_time(e1) / 1e3)
    plan.status()
    return float(np.median(times))


def autotune(m_per_sys, n_per_sys, packed_or_user, precision: str = "fp64", cache: Path | str | None = None,
             use_cache: bool = True, log=None) -> dict:
    """Pick seg_len[m] per block size present and warps_per_cta for this
    batch's (m, N, nsys) bucket by timing the real batch: coordinate descent
    over SEG_CANDIDATES for each m (largest m first), then WARP_CANDIDATES.
    ``packed_or_user``: per-system (ua, ub, uc, ud) device tensors.  The packed
    layout does not depend on the tuning, so it is packed once.  Results are
    cached by bucket in a JSON file."""
    cache = Path(cache) if cache else default_cache()
    key = bucket_key(m_per_sys, n_per_sys, precision)
    store = {}
    if cache.exists():
        try:
            store = json.loads(cache.read_text())
        except (OSError, ValueError):
            store = {}
    if use_cache and key in store:
        hit = store[key]
        return {"seg_len": {int(k): int(v) for k, v in hit["seg_len"].items()},
                "warps_per_cta": int(hit["warps_per_cta"]), "ms": float(hit["ms"])}
    ua, ub, uc, ud = packed_or_user
    ms = sorted({int(x) for x in np.unique(m_per_sys)}, reverse=True)
    best = {"seg_len": {m: 256 for m in ms}, "warps_per_cta": 4}
    probe = BatchPlan(m_per_sys, n_per_sys, precision, best)
    packed = probe.pack(ua, ub, uc, ud)
    d0 = packed[3].clone()
    probe.destroy()

    def trial(cfg):
        plan = BatchPlan(m_per_sys, n_per_sys, precision, cfg)
        t = time_solve(plan, packed, d0)
        plan.destroy()
        if log:
            log(f"autotune {cfg}: {t * 1e3:.3f} ms")
        return t

    best_t = trial(best)
    for m in ms:
        for L in SEG_CANDIDATES:
            if L == best["seg_len"][m]:
                continue
            cfg = {"seg_len": {**best["seg_len"], m: L}, "warps_per_cta": best["warps_per_cta"]}
            t = trial(cfg)
            if t < best_t:
                best, best_t = cfg, t
    for w in WARP_CANDIDATES:
        if w == best["warps_per_cta"]:
            continue
        cfg = {"seg_len": best["seg_len"], "warps_per_cta": w}
        t = trial(cfg)
        if t < best_t:
            best, best_t = cfg, t
    best = {"seg_len": {int(k): int(v) for k, v in best["seg_len"].items()}, "warps_per_cta": best["warps_per_cta"],
            "ms": best_t * 1e3}
    store[key] = best
    try:
        cache.parent.mkdir(parents=True, exist_ok=True)
        cache.write_text(json.dumps(store, indent=1, sort_keys=True))
    except OSError:
        pass
    return best


def capture_sweeps(plan: BatchPlan, packed, d0, sweeps: int = 100):
    """A CUDA graph of `sweeps` sweeps, each restoring D from d0 and solving.
    Returns the graph (replay with .replay())."""
    import torch

    pa, pb, pc, pd = packed
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):  # warm-up outside capture
        pd.copy_(d0)
        plan.solve(pa, pb, pc, pd, stream=s)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        for _ in range(sweeps):
            pd.copy_(d0)
            plan.solve(pa, pb, pc, pd)
    return g
