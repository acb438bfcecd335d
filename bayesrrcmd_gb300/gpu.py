"""ctypes binding of libbrr_gpu.so (the C ABI declared in include/brr_gpu.h).

This is the Python mirror of the host interface the reference exposes for the
BayesR path (src/analysis.h:25-52, src/markerbuilder.h:11-42): pack the
markers, set groups and phenotype, initialise, run the Gibbs chain, read the
state.  It is a thin binding: all compute runs in the CUDA library, and
loading fails loudly when the library is missing.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

MAX_GROUPS = 64
MAX_K = 16

KIND_DENSE, KIND_RAGGED, KIND_EIGEN = 0, 1, 2
FORM_FP64, FORM_FP32C = 0, 1

ERRORS = {
    -1: "BRR_ERR_ARG", -2: "BRR_ERR_CUDA", -3: "BRR_ERR_OOM", -4: "BRR_ERR_TIMEOUT",
    -5: "BRR_ERR_MARKER", -6: "BRR_ERR_RANGE", -7: "BRR_ERR_STREAM", -8: "BRR_ERR_DEVICE",
}


class BrrConfig(C.Structure):
    _fields_ = [
        ("N", C.c_int64), ("M", C.c_int64), ("kind", C.c_int32), ("form", C.c_int32),
        ("n_groups", C.c_int32), ("K", C.c_int32 * MAX_GROUPS),
        ("S", C.c_double * (MAX_GROUPS * (MAX_K - 1))),
        ("seed", C.c_uint32), ("chain", C.c_uint32),
        ("v0E", C.c_double), ("s02E", C.c_double), ("v0G", C.c_double), ("s02G", C.c_double),
        ("refresh_every", C.c_int32), ("spec_width", C.c_int32), ("grid", C.c_int32), ("device", C.c_int32),
        ("gram", C.c_int32), ("async_batch", C.c_int32), ("cluster", C.c_int32), ("pair_rounds", C.c_int32),
    ]


class BrrState(C.Structure):
    _fields_ = [
        ("beta", C.POINTER(C.c_double)), ("comp", C.POINTER(C.c_int32)), ("acum", C.POINTER(C.c_double)),
        ("eps", C.POINTER(C.c_double)), ("mu", C.c_double), ("sigmaE", C.c_double), ("epsSum", C.c_double),
        ("sigmaG", C.c_double * MAX_GROUPS), ("pi", C.c_double * (MAX_GROUPS * MAX_K)), ("iteration", C.c_uint32),
    ]


class BrrSweepOut(C.Structure):
    _fields_ = [
        ("v", C.c_double * (MAX_GROUPS * MAX_K)), ("betasqnG", C.c_double * MAX_GROUPS),
        ("eps_sqnorm", C.c_double), ("eps_sum", C.c_double), ("rounds", C.c_int64),
    ]


_LIB: Optional[C.CDLL] = None
LIB_PATH = Path(__file__).resolve().parent / "lib" / "libbrr_gpu.so"

EXPORTS = [
    "brr_last_error", "brr_ctx_create", "brr_ctx_destroy", "brr_pack_bed", "brr_pack_bed_device",
    "brr_get_marker_table", "brr_get_ragged_lists", "brr_set_groups", "brr_set_phenotype", "brr_init_chain",
    "brr_iterate", "brr_sweep", "brr_get_state", "brr_set_state", "brr_refresh_eps", "brr_get_timing", "brr_get_phase_cycles",
    "brr_set_wait_limit", "brr_set_profiling", "brr_xbeta", "brr_synth_bed_device", "brr_xbeta_noalloc",
    "brr_get_gram_info",
    "brr_get_gram_entries",
    "brr_get_round_info",
    "brr_get_gram_bits",
    "brr_batch_create", "brr_batch_destroy", "brr_batch_pack_bed", "brr_batch_pack_bed_device",
    "brr_batch_set_groups", "brr_batch_set_phenotypes", "brr_batch_init", "brr_batch_iterate",
    "brr_batch_get_chain_state", "brr_batch_get_timing", "brr_batch_set_wait_limit", "brr_batch_set_profiling",
    "brr_batch_get_geometry",
    "brr_multi_create", "brr_multi_destroy", "brr_multi_pack_bed", "brr_multi_pack_bed_device",
    "brr_multi_set_groups", "brr_multi_set_phenotype", "brr_multi_init", "brr_multi_tune", "brr_multi_iterate",
    "brr_multi_get_state", "brr_multi_get_timing", "brr_synth_bed_device_beta", "brr_multi_set_wait_limit",
    "brr_get_sweep_timeline",
]


def load_library(path: Optional[Path] = None) -> C.CDLL:
    """Load libbrr_gpu.so; raises if it has not been built (no fallback)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -m bayesrrcmd_gb300.build` "
                           "(the GPU path has no CPU fallback)")
    lib = C.CDLL(str(p))
    P = C.c_void_p
    lib.brr_last_error.restype = C.c_char_p
    lib.brr_ctx_create.argtypes = [C.POINTER(BrrConfig), C.POINTER(P)]
    lib.brr_ctx_destroy.argtypes = [P]
    lib.brr_pack_bed.argtypes = [P, C.POINTER(C.c_uint8), C.c_int64]
    lib.brr_pack_bed_device.argtypes = [P, P, C.c_int64]
    lib.brr_get_marker_table.argtypes = [P, C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    lib.brr_get_ragged_lists.argtypes = [P] + [C.POINTER(C.c_int64), C.POINTER(C.c_int32)] * 3
    lib.brr_set_groups.argtypes = [P, C.POINTER(C.c_int32)]
    lib.brr_set_phenotype.argtypes = [P, C.POINTER(C.c_float)]
    lib.brr_init_chain.argtypes = [P]
    lib.brr_iterate.argtypes = [P, C.c_int32]
    lib.brr_sweep.argtypes = [P, C.POINTER(C.c_uint32), C.POINTER(C.c_double), C.POINTER(C.c_double),
                              C.POINTER(BrrSweepOut)]
    lib.brr_get_state.argtypes = [P, C.POINTER(BrrState)]
    lib.brr_set_state.argtypes = [P, C.POINTER(BrrState)]
    lib.brr_refresh_eps.argtypes = [P]
    lib.brr_get_timing.argtypes = [P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    lib.brr_get_phase_cycles.argtypes = [P, C.POINTER(C.c_int64)]
    lib.brr_set_wait_limit.argtypes = [P, C.c_uint64, C.c_int32]
    lib.brr_set_profiling.argtypes = [P, C.c_int32]
    lib.brr_get_sweep_timeline.argtypes = [P, C.POINTER(C.c_uint64), C.c_int64, C.POINTER(C.c_int32),
                                           C.POINTER(C.c_int32)]
    lib.brr_get_gram_info.argtypes = [P, C.POINTER(C.c_int32), C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    lib.brr_get_gram_entries.argtypes = [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_int64,
                                         C.POINTER(C.c_double)]
    lib.brr_get_round_info.argtypes = [P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    lib.brr_get_gram_bits.argtypes = [P, C.POINTER(C.c_int32)]
    lib.brr_xbeta.argtypes = [P, C.POINTER(C.c_uint32), C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_double)]
    lib.brr_xbeta_noalloc.argtypes = [P, C.POINTER(C.c_uint32), C.POINTER(C.c_double), C.c_int64, P]
    lib.brr_synth_bed_device.argtypes = [P, C.c_int64, C.c_int64, C.c_uint32, C.c_double, C.c_double, C.c_double]
    lib.brr_synth_bed_device_beta.argtypes = [P, C.c_int64, C.c_int64, C.c_uint32, C.c_double, C.c_double,
                                              C.c_double, C.c_double, C.c_double]
    lib.brr_batch_create.argtypes = [C.POINTER(BrrConfig), C.c_int32, C.POINTER(P)]
    lib.brr_batch_destroy.argtypes = [P]
    lib.brr_batch_pack_bed.argtypes = [P, C.POINTER(C.c_uint8), C.c_int64]
    lib.brr_batch_pack_bed_device.argtypes = [P, P, C.c_int64]
    lib.brr_batch_set_groups.argtypes = [P, C.POINTER(C.c_int32)]
    lib.brr_batch_set_phenotypes.argtypes = [P, C.POINTER(C.c_float)]
    lib.brr_batch_init.argtypes = [P]
    lib.brr_batch_iterate.argtypes = [P, C.c_int32]
    lib.brr_batch_get_chain_state.argtypes = [P, C.c_int32, C.POINTER(BrrState)]
    lib.brr_batch_get_timing.argtypes = [P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    lib.brr_batch_set_wait_limit.argtypes = [P, C.c_uint64, C.c_int32]
    lib.brr_batch_set_profiling.argtypes = [P, C.c_int32]
    lib.brr_batch_get_geometry.argtypes = [P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
    lib.brr_multi_create.argtypes = [C.POINTER(BrrConfig), C.c_int32, C.POINTER(P)]
    lib.brr_multi_destroy.argtypes = [P]
    lib.brr_multi_pack_bed.argtypes = [P, C.c_int32, C.POINTER(C.c_uint8), C.c_int64]
    lib.brr_multi_pack_bed_device.argtypes = [P, C.c_int32, P, C.c_int64]
    lib.brr_multi_set_groups.argtypes = [P, C.c_int32, C.POINTER(C.c_int32)]
    lib.brr_multi_set_phenotype.argtypes = [P, C.c_int32, C.POINTER(C.c_float)]
    lib.brr_multi_init.argtypes = [P]
    lib.brr_multi_tune.argtypes = [P, C.c_int32]
    lib.brr_multi_iterate.argtypes = [P, C.c_int32]
    lib.brr_multi_get_state.argtypes = [P, C.c_int32, C.POINTER(BrrState)]
    lib.brr_multi_set_wait_limit.argtypes = [P, C.c_int32, C.c_uint64, C.c_int32]
    lib.brr_multi_get_timing.argtypes = [P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int32),
                                         C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    for name in EXPORTS:
        if name != "brr_last_error":
            getattr(lib, name).restype = C.c_int
    if path is None:
        _LIB = lib
    return lib


def synth_bed_device(dev_ptr: int, N: int, M: int, seed: int, p_lo: float, p_hi: float, missing: float = 0.0,
                     lib: Optional[C.CDLL] = None):
    """Fill a device buffer of M*ceil(N/4) bytes with a seeded synthetic BED payload."""
    lib = lib or load_library()
    rc = lib.brr_synth_bed_device(C.c_void_p(dev_ptr), N, M, seed & 0xFFFFFFFF, p_lo, p_hi, missing)
    if rc != 0:
        raise BrrError(rc, lib.brr_last_error().decode())


def synth_bed_device_beta(dev_ptr: int, N: int, M: int, seed: int, a: float, b: float, p_lo: float, p_hi: float,
                          missing: float = 0.0, lib: Optional[C.CDLL] = None):
    """As synth_bed_device with allele frequencies ~ Beta(a, b) clipped to [p_lo, p_hi]."""
    lib = lib or load_library()
    rc = lib.brr_synth_bed_device_beta(C.c_void_p(dev_ptr), N, M, seed & 0xFFFFFFFF, a, b, p_lo, p_hi, missing)
    if rc != 0:
        raise BrrError(rc, lib.brr_last_error().decode())


class BrrError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def _ptr(a: np.ndarray, ct):
    return a.ctypes.data_as(C.POINTER(ct))


@dataclass
class ChainConfig:
    """Mirror of the reference Options used on this path (src/options.hpp:21-105)."""
    N: int
    M: int
    kind: int = KIND_DENSE
    form: int = FORM_FP64
    S: Sequence[Sequence[float]] = field(default_factory=lambda: [[0.01, 0.001, 0.0001]])
    seed: int = 1
    chain: int = 0
    v0E: float = 1e-4
    s02E: float = 1e-4
    v0G: float = 1e-4
    s02G: float = 1e-4
    refresh_every: int = 0
    spec_width: int = 0
    grid: int = 0
    device: int = 0
    gram: int = 0
    async_batch: int = 0
    cluster: int = 0
    pair_rounds: int = 0

    def to_c(self) -> BrrConfig:
        c = BrrConfig()
        c.N, c.M, c.kind, c.form = self.N, self.M, self.kind, self.form
        c.n_groups = len(self.S)
        for g, row in enumerate(self.S):
            c.K[g] = len(row) + 1
            for k, v in enumerate(row):
                c.S[g * (MAX_K - 1) + k] = float(v)
        c.seed, c.chain = self.seed & 0xFFFFFFFF, self.chain & 0xFFFFFFFF
        c.v0E, c.s02E, c.v0G, c.s02G = self.v0E, self.s02E, self.v0G, self.s02G
        c.refresh_every, c.spec_width, c.grid, c.device = self.refresh_every, self.spec_width, self.grid, self.device
        c.gram = self.gram
        c.async_batch = self.async_batch
        c.cluster = self.cluster
        c.pair_rounds = self.pair_rounds
        return c


class Chain:
    """One BayesR Markov chain on one GPU, behind the C ABI."""

    def __init__(self, cfg: ChainConfig, lib: Optional[C.CDLL] = None):
        self.cfg = cfg
        self.lib = lib or load_library()
        self._c = cfg.to_c()
        h = C.c_void_p()
        self._check(self.lib.brr_ctx_create(C.byref(self._c), C.byref(h)))
        self.h = h

    def _check(self, rc: int):
        if rc != 0:
            raise BrrError(rc, self.lib.brr_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.brr_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # preprocess ------------------------------------------------------------
    def pack_bed(self, bed_payload: np.ndarray):
        a = np.ascontiguousarray(bed_payload, dtype=np.uint8)
        self._check(self.lib.brr_pack_bed(self.h, _ptr(a, C.c_uint8), a.size))

    def pack_bed_device(self, dev_ptr: int, nbytes: int):
        self._check(self.lib.brr_pack_bed_device(self.h, C.c_void_p(dev_ptr), nbytes))

    def marker_table(self):
        t = np.zeros((self.cfg.M, 4), np.float64)
        n = np.zeros((self.cfg.M, 4), np.int64)
        self._check(self.lib.brr_get_marker_table(self.h, _ptr(t, C.c_double), _ptr(n, C.c_int64)))
        return t, n

    def ragged_lists(self, counts: np.ndarray):
        M = self.cfg.M
        offs = [np.zeros(M + 1, np.int64) for _ in range(3)]
        tot = [int(counts[:, 1].sum()), int(counts[:, 2].sum()), int(counts[:, 3].sum())]
        idx = [np.zeros(max(t, 1), np.int32) for t in tot]
        args = []
        for k in range(3):
            args += [_ptr(offs[k], C.c_int64), _ptr(idx[k], C.c_int32)]
        self._check(self.lib.brr_get_ragged_lists(self.h, *args))
        return [(offs[k], idx[k][:tot[k]]) for k in range(3)]

    # chain -----------------------------------------------------------------
    def set_groups(self, group: np.ndarray):
        g = np.ascontiguousarray(group, dtype=np.int32)
        self._check(self.lib.brr_set_groups(self.h, _ptr(g, C.c_int32)))

    def set_phenotype(self, y: np.ndarray):
        a = np.ascontiguousarray(y, dtype=np.float32)
        self._check(self.lib.brr_set_phenotype(self.h, _ptr(a, C.c_float)))

    def init(self):
        self._check(self.lib.brr_init_chain(self.h))

    def iterate(self, n: int = 1):
        self._check(self.lib.brr_iterate(self.h, int(n)))

    def sweep(self, order: np.ndarray, u: np.ndarray, z: np.ndarray) -> BrrSweepOut:
        o = np.ascontiguousarray(order, dtype=np.uint32)
        uu = np.ascontiguousarray(u, dtype=np.float64)
        zz = np.ascontiguousarray(z, dtype=np.float64)
        out = BrrSweepOut()
        self._check(self.lib.brr_sweep(self.h, _ptr(o, C.c_uint32), _ptr(uu, C.c_double), _ptr(zz, C.c_double),
                                       C.byref(out)))
        return out

    def refresh(self):
        self._check(self.lib.brr_refresh_eps(self.h))

    def state(self) -> dict:
        M, N = self.cfg.M, self.cfg.N
        beta = np.zeros(M, np.float64)
        comp = np.zeros(M, np.int32)
        acum = np.zeros(M, np.float64)
        eps = np.zeros(N, np.float64)
        st = BrrState()
        st.beta, st.comp, st.acum, st.eps = (_ptr(beta, C.c_double), _ptr(comp, C.c_int32),
                                             _ptr(acum, C.c_double), _ptr(eps, C.c_double))
        self._check(self.lib.brr_get_state(self.h, C.byref(st)))
        G = len(self.cfg.S)
        return dict(beta=beta, comp=comp, acum=acum, eps=eps, mu=st.mu, sigmaE=st.sigmaE, epsSum=st.epsSum,
                    sigmaG=np.array(st.sigmaG[:G]),
                    pi=np.array(st.pi[:]).reshape(MAX_GROUPS, MAX_K)[:G].copy(), iteration=st.iteration)

    def set_state(self, s: dict):
        beta = np.ascontiguousarray(s["beta"], np.float64)
        comp = np.ascontiguousarray(s["comp"], np.int32)
        acum = np.ascontiguousarray(s["acum"], np.float64)
        eps = np.ascontiguousarray(s["eps"], np.float64)
        st = BrrState()
        st.beta, st.comp, st.acum, st.eps = (_ptr(beta, C.c_double), _ptr(comp, C.c_int32),
                                             _ptr(acum, C.c_double), _ptr(eps, C.c_double))
        st.mu, st.sigmaE, st.epsSum = s["mu"], s["sigmaE"], s.get("epsSum", 0.0)
        for g, v in enumerate(s["sigmaG"]):
            st.sigmaG[g] = v
        pi = np.asarray(s["pi"])
        for g in range(pi.shape[0]):
            for k in range(pi.shape[1]):
                st.pi[g * MAX_K + k] = pi[g, k]
        st.iteration = int(s.get("iteration", 0))
        self._check(self.lib.brr_set_state(self.h, C.byref(st)))

    def xbeta(self, idx: np.ndarray, b: np.ndarray) -> np.ndarray:
        i = np.ascontiguousarray(idx, np.uint32)
        bb = np.ascontiguousarray(b, np.float64)
        out = np.zeros(self.cfg.N, np.float64)
        self._check(self.lib.brr_xbeta(self.h, _ptr(i, C.c_uint32), _ptr(bb, C.c_double), i.size,
                                       _ptr(out, C.c_double)))
        return out

    def set_wait_limit(self, timeout_ns: int, phantom_arrivals: int = 0):
        self._check(self.lib.brr_set_wait_limit(self.h, int(timeout_ns), int(phantom_arrivals)))

    def set_profiling(self, on):
        """Phase counters (phase_cycles) on or off; 2 adds the blocked sweep's
        per-CTA event timeline (timeline()); timed runs keep them off."""
        self._check(self.lib.brr_set_profiling(self.h, int(on) if not isinstance(on, bool) else (1 if on else 0)))

    def timeline(self) -> np.ndarray:
        """Events [iteration, cta, event] (global timer, ns) of the last sweep
        run with profiling 2."""
        ev = 16
        n = 64 * 152 * ev * 2
        buf = np.zeros(n, np.uint64)
        it, ctas = C.c_int32(), C.c_int32()
        self._check(self.lib.brr_get_sweep_timeline(self.h, _ptr(buf, C.c_uint64), n, C.byref(it), C.byref(ctas)))
        return buf[:it.value * ctas.value * ev].reshape(it.value, ctas.value, ev).copy()

    def gram_entries(self, j, k) -> np.ndarray:
        j = np.ascontiguousarray(j, np.int64)
        k = np.ascontiguousarray(k, np.int64)
        out = np.zeros(j.size, np.float64)
        self._check(self.lib.brr_get_gram_entries(self.h, _ptr(j, C.c_int64), _ptr(k, C.c_int64), j.size,
                                                  _ptr(out, C.c_double)))
        return out

    def round_info(self):
        pr, last = C.c_int32(), C.c_int32()
        self._check(self.lib.brr_get_round_info(self.h, C.byref(pr), C.byref(last)))
        return dict(pair_rounds=bool(pr.value), last_sweep_pair_rounds=bool(last.value))

    def gram_info(self):
        b, ms, n, bits = C.c_int32(), C.c_double(), C.c_int64(), C.c_int32()
        self._check(self.lib.brr_get_gram_info(self.h, C.byref(b), C.byref(ms), C.byref(n)))
        self._check(self.lib.brr_get_gram_bits(self.h, C.byref(bits)))
        return dict(blocked=bool(b.value), build_ms=ms.value, bytes=n.value, operand_bits=bits.value)

    def phase_cycles(self) -> np.ndarray:
        out = np.zeros(16, np.int64)
        self._check(self.lib.brr_get_phase_cycles(self.h, _ptr(out, C.c_int64)))
        return out

    def timing(self):
        sw, tot, r = C.c_double(), C.c_double(), C.c_int64()
        self._check(self.lib.brr_get_timing(self.h, C.byref(sw), C.byref(tot), C.byref(r)))
        return sw.value, tot.value, r.value


class Batch:
    """C = 32 or 64 chains (distinct seeds cfg.chain .. cfg.chain+C-1, one
    phenotype each) on shared dense genotypes, swept together with the
    tensor-core batched form behind the C ABI."""

    def __init__(self, cfg: ChainConfig, chains: int, lib: Optional[C.CDLL] = None):
        self.cfg = cfg
        self.C = int(chains)
        self.lib = lib or load_library()
        self._c = cfg.to_c()
        h = C.c_void_p()
        self._check(self.lib.brr_batch_create(C.byref(self._c), self.C, C.byref(h)))
        self.h = h

    def _check(self, rc: int):
        if rc != 0:
            raise BrrError(rc, self.lib.brr_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.brr_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def pack_bed(self, bed_payload: np.ndarray):
        a = np.ascontiguousarray(bed_payload, dtype=np.uint8)
        self._check(self.lib.brr_batch_pack_bed(self.h, _ptr(a, C.c_uint8), a.size))

    def pack_bed_device(self, dev_ptr: int, nbytes: int):
        self._check(self.lib.brr_batch_pack_bed_device(self.h, C.c_void_p(dev_ptr), nbytes))

    def set_groups(self, group: np.ndarray):
        g = np.ascontiguousarray(group, dtype=np.int32)
        self._check(self.lib.brr_batch_set_groups(self.h, _ptr(g, C.c_int32)))

    def set_phenotypes(self, y: np.ndarray):
        a = np.ascontiguousarray(y, dtype=np.float32)
        if a.shape != (self.C, self.cfg.N):
            raise ValueError(f"phenotypes must be {self.C} x {self.cfg.N}")
        self._check(self.lib.brr_batch_set_phenotypes(self.h, _ptr(a, C.c_float)))

    def init(self):
        self._check(self.lib.brr_batch_init(self.h))

    def iterate(self, n: int = 1):
        self._check(self.lib.brr_batch_iterate(self.h, int(n)))

    def state(self, chain: int) -> dict:
        M, N = self.cfg.M, self.cfg.N
        beta = np.zeros(M, np.float64)
        comp = np.zeros(M, np.int32)
        acum = np.zeros(M, np.float64)
        eps = np.zeros(N, np.float64)
        st = BrrState()
        st.beta, st.comp, st.acum, st.eps = (_ptr(beta, C.c_double), _ptr(comp, C.c_int32),
                                             _ptr(acum, C.c_double), _ptr(eps, C.c_double))
        self._check(self.lib.brr_batch_get_chain_state(self.h, int(chain), C.byref(st)))
        G = len(self.cfg.S)
        return dict(beta=beta, comp=comp, acum=acum, eps=eps, mu=st.mu, sigmaE=st.sigmaE, epsSum=st.epsSum,
                    sigmaG=np.array(st.sigmaG[:G]),
                    pi=np.array(st.pi[:]).reshape(MAX_GROUPS, MAX_K)[:G].copy(), iteration=st.iteration)

    def timing(self):
        sw, tot = C.c_double(), C.c_double()
        cyc = np.zeros(8, np.int64)
        self._check(self.lib.brr_batch_get_timing(self.h, C.byref(sw), C.byref(tot), _ptr(cyc, C.c_int64)))
        return sw.value, tot.value, cyc

    def set_wait_limit(self, timeout_ns: int, phantom_arrivals: int = 0):
        self._check(self.lib.brr_batch_set_wait_limit(self.h, int(timeout_ns), int(phantom_arrivals)))

    def set_profiling(self, on: bool):
        """Phase counters (timing()'s cycles) on or off; timed runs keep them off."""
        self._check(self.lib.brr_batch_set_profiling(self.h, 1 if on else 0))

    def geometry(self):
        g, sl, sm = C.c_int32(), C.c_int32(), C.c_int64()
        self._check(self.lib.brr_batch_get_geometry(self.h, C.byref(g), C.byref(sl), C.byref(sm)))
        return dict(ctas=g.value, slice=sl.value, smem=sm.value)


class Multi:
    """Independent regressions of different sizes (each its own ChainConfig:
    N, M, kind, groups, S, seed, chain; one sweep form) swept together, one
    cooperative launch per iteration, behind the C ABI."""

    def __init__(self, cfgs: Sequence[ChainConfig], lib: Optional[C.CDLL] = None):
        self.cfgs = list(cfgs)
        self.n = len(self.cfgs)
        self.lib = lib or load_library()
        arr = (BrrConfig * self.n)(*[c.to_c() for c in self.cfgs])
        self._arr = arr
        h = C.c_void_p()
        self._check(self.lib.brr_multi_create(arr, self.n, C.byref(h)))
        self.h = h

    def _check(self, rc: int):
        if rc != 0:
            raise BrrError(rc, self.lib.brr_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.brr_multi_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def pack_bed(self, i: int, bed_payload: np.ndarray):
        a = np.ascontiguousarray(bed_payload, dtype=np.uint8)
        self._check(self.lib.brr_multi_pack_bed(self.h, int(i), _ptr(a, C.c_uint8), a.size))

    def pack_bed_device(self, i: int, dev_ptr: int, nbytes: int):
        self._check(self.lib.brr_multi_pack_bed_device(self.h, int(i), C.c_void_p(dev_ptr), nbytes))

    def set_groups(self, i: int, group: np.ndarray):
        g = np.ascontiguousarray(group, dtype=np.int32)
        self._check(self.lib.brr_multi_set_groups(self.h, int(i), _ptr(g, C.c_int32)))

    def set_phenotype(self, i: int, y: np.ndarray):
        a = np.ascontiguousarray(y, dtype=np.float32)
        self._check(self.lib.brr_multi_set_phenotype(self.h, int(i), _ptr(a, C.c_float)))

    def init(self):
        self._check(self.lib.brr_multi_init(self.h))

    def tune(self, rounds: int = 2):
        self._check(self.lib.brr_multi_tune(self.h, int(rounds)))

    def iterate(self, n: int = 1):
        self._check(self.lib.brr_multi_iterate(self.h, int(n)))

    def set_wait_limit(self, timeout_ns: int, phantom_arrivals: int = 0, instance: int = -1):
        self._check(self.lib.brr_multi_set_wait_limit(self.h, int(instance), int(timeout_ns), int(phantom_arrivals)))

    def state(self, i: int) -> dict:
        cfg = self.cfgs[i]
        M, N = cfg.M, cfg.N
        beta = np.zeros(M, np.float64)
        comp = np.zeros(M, np.int32)
        acum = np.zeros(M, np.float64)
        eps = np.zeros(N, np.float64)
        st = BrrState()
        st.beta, st.comp, st.acum, st.eps = (_ptr(beta, C.c_double), _ptr(comp, C.c_int32),
                                             _ptr(acum, C.c_double), _ptr(eps, C.c_double))
        self._check(self.lib.brr_multi_get_state(self.h, int(i), C.byref(st)))
        G = len(cfg.S)
        return dict(beta=beta, comp=comp, acum=acum, eps=eps, mu=st.mu, sigmaE=st.sigmaE, epsSum=st.epsSum,
                    sigmaG=np.array(st.sigmaG[:G]),
                    pi=np.array(st.pi[:]).reshape(MAX_GROUPS, MAX_K)[:G].copy(), iteration=st.iteration)

    def timing(self):
        sw, tot = C.c_double(), C.c_double()
        ctas = np.zeros(self.n, np.int32)
        width = np.zeros(self.n, np.int32)
        ms = np.zeros(self.n, np.float64)
        self._check(self.lib.brr_multi_get_timing(self.h, C.byref(sw), C.byref(tot), _ptr(ctas, C.c_int32),
                                                  _ptr(width, C.c_int32), _ptr(ms, C.c_double)))
        return dict(sweep_ms=sw.value, total_ms=tot.value, ctas=ctas, width=width, inst_ms=ms)
