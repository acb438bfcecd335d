"""ctypes binding of the CPU oracle (oracle/liboracle.so), used only as the checker."""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

from oracle.build import build_oracle, build_oracle_timing  # noqa: E402

OR_MAX_GROUPS = 64
OR_MAX_K = 16


class OrProblem(C.Structure):
    _fields_ = [
        ("N", C.c_int64), ("M", C.c_int64), ("kind", C.c_int32), ("n_groups", C.c_int32),
        ("group", C.POINTER(C.c_int32)), ("K", C.POINTER(C.c_int32)), ("S", C.POINTER(C.c_double)),
        ("y", C.POINTER(C.c_float)), ("bed", C.POINTER(C.c_uint8)), ("seed", C.c_uint32), ("chain", C.c_uint32),
        ("v0E", C.c_double), ("s02E", C.c_double), ("v0G", C.c_double), ("s02G", C.c_double),
        ("shared_perm", C.c_int32), ("perm_chain", C.c_uint32), ("dense_lut", C.c_int32),
        ("async_batch", C.c_int32),
    ]


class OrState(C.Structure):
    _fields_ = [
        ("beta", C.POINTER(C.c_double)), ("comp", C.POINTER(C.c_int32)), ("acum", C.POINTER(C.c_double)),
        ("eps", C.POINTER(C.c_double)), ("mu", C.c_double), ("sigmaE", C.c_double), ("epsSum", C.c_double),
        ("sigmaG", C.c_double * OR_MAX_GROUPS), ("pi", C.c_double * (OR_MAX_GROUPS * OR_MAX_K)),
        ("v", C.c_double * (OR_MAX_GROUPS * OR_MAX_K)), ("betasqnG", C.c_double * OR_MAX_GROUPS), ("m0", C.c_double),
    ]


_lib = None
_timing = False


def use_timing_build():
    """Load the oracle built with the reference's fast release flags from now
    on in this process: for the timed CPU baseline only, never as the checker."""
    global _lib, _timing
    if not _timing:
        _timing = True
        _lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(str(build_oracle_timing() if _timing else build_oracle()))
        u8, i8, i32, i64, f64, u32 = (C.POINTER(C.c_uint8), C.POINTER(C.c_int8), C.POINTER(C.c_int32),
                                      C.POINTER(C.c_int64), C.POINTER(C.c_double), C.POINTER(C.c_uint32))
        L.or_philox4x32_10.argtypes = [u32, u32, u32]
        L.or_u53.argtypes = [C.c_uint32, C.c_uint32]
        L.or_u53.restype = C.c_double
        L.or_marker_draws.argtypes = [C.c_uint32] * 4 + [f64, f64]
        L.or_permutation.argtypes = [C.c_uint32] * 4 + [u32]
        L.or_gamma.argtypes = [C.c_uint32] * 5 + [C.c_double, f64]
        L.or_decode_bed.argtypes = [u8, C.c_int64, C.c_int64, i8]
        L.or_marker_counts.argtypes = [u8, C.c_int64, C.c_int64, i64]
        L.or_dense_lut.argtypes = [u8, C.c_int64, C.c_int64, f64]
        L.or_dense_columns.argtypes = [u8, C.c_int64, C.c_int64, f64]
        L.or_ragged_stats.argtypes = [u8, C.c_int64, C.c_int64, f64]
        L.or_eigen_stats.argtypes = [u8, C.c_int64, C.c_int64, f64]
        L.or_ragged_lists.argtypes = [u8, C.c_int64, C.c_int64, i64, i32, i64, i32, i64, i32]
        L.or_markers_create.argtypes = [C.POINTER(OrProblem), C.POINTER(C.c_void_p)]
        L.or_markers_destroy.argtypes = [C.c_void_p]
        L.or_init.argtypes = [C.POINTER(OrProblem), C.POINTER(OrState)]
        L.or_iterate.argtypes = [C.POINTER(OrProblem), C.c_void_p, C.POINTER(OrState), C.c_uint32]
        L.or_sweep.argtypes = [C.POINTER(OrProblem), C.c_void_p, C.POINTER(OrState), u32, f64, f64]
        _lib = L
    return _lib


def p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def philox(ctr, key):
    c = np.array(ctr, np.uint32)
    k = np.array(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib().or_philox4x32_10(p(c, C.c_uint32), p(k, C.c_uint32), p(o, C.c_uint32))
    return [int(x) for x in o]


def marker_table_dense(bed, N):
    M = bed.shape[0]
    out = np.zeros((M, 4))
    rc = lib().or_dense_lut(p(np.ascontiguousarray(bed), C.c_uint8), N, M, p(out, C.c_double))
    return rc, out


def dense_columns(bed, N):
    M = bed.shape[0]
    out = np.zeros((M, N))
    rc = lib().or_dense_columns(p(np.ascontiguousarray(bed), C.c_uint8), N, M, p(out, C.c_double))
    assert rc == 0
    return out


def counts(bed, N):
    M = bed.shape[0]
    out = np.zeros((M, 4), np.int64)
    assert lib().or_marker_counts(p(np.ascontiguousarray(bed), C.c_uint8), N, M, p(out, C.c_int64)) == 0
    return out


def ragged_stats(bed, N):
    M = bed.shape[0]
    out = np.zeros((M, 4))
    rc = lib().or_ragged_stats(p(np.ascontiguousarray(bed), C.c_uint8), N, M, p(out, C.c_double))
    return rc, out


def eigen_stats(bed, N):
    M = bed.shape[0]
    out = np.zeros((M, 4))
    rc = lib().or_eigen_stats(p(np.ascontiguousarray(bed), C.c_uint8), N, M, p(out, C.c_double))
    return rc, out


def ragged_lists(bed, N):
    M = bed.shape[0]
    c = counts(bed, N)
    offs = [np.zeros(M + 1, np.int64) for _ in range(3)]
    idx = [np.zeros(max(int(c[:, k].sum()), 1), np.int32) for k in (1, 2, 3)]
    args = []
    for k in range(3):
        args += [p(offs[k], C.c_int64), p(idx[k], C.c_int32)]
    assert lib().or_ragged_lists(p(np.ascontiguousarray(bed), C.c_uint8), N, M, *args) == 0
    return [(offs[k], idx[k][:int(c[:, k + 1].sum())]) for k in range(3)]


def decode(bed, N):
    M = bed.shape[0]
    out = np.zeros((M, N), np.int8)
    assert lib().or_decode_bed(p(np.ascontiguousarray(bed), C.c_uint8), N, M, p(out, C.c_int8)) == 0
    return out


def permutation(seed, chain, it, M):
    out = np.zeros(M, np.uint32)
    lib().or_permutation(seed, chain, it, M, p(out, C.c_uint32))
    return out


def marker_draws(seed, chain, it, M):
    u = np.zeros(M)
    z = np.zeros(M)
    uu, zz = C.c_double(), C.c_double()
    for j in range(M):
        lib().or_marker_draws(seed, chain, it, j, C.byref(uu), C.byref(zz))
        u[j], z[j] = uu.value, zz.value
    return u, z


def gamma(seed, chain, it, purpose, sub, shape):
    out = C.c_double()
    rc = lib().or_gamma(seed, chain, it, purpose, sub, shape, C.byref(out))
    return rc, out.value


class OracleChain:
    """Oracle chain over the same inputs as the GPU Chain."""

    def __init__(self, bed, N, y, S, kind=0, group=None, seed=1, chain=0, priors=(1e-4, 1e-4, 1e-4, 1e-4),
                 perm_chain=None, dense_lut=False, async_batch=0):
        self.bed = np.ascontiguousarray(bed, np.uint8)
        self.N, self.M = N, bed.shape[0]
        self.y = np.ascontiguousarray(y, np.float32)
        G = len(S)
        self.G = G
        self.group = np.ascontiguousarray(group if group is not None else np.zeros(self.M), np.int32)
        self.K = np.array([len(r) + 1 for r in S], np.int32)
        self.S = np.zeros(G * (OR_MAX_K - 1))
        for g, r in enumerate(S):
            self.S[g * (OR_MAX_K - 1):g * (OR_MAX_K - 1) + len(r)] = r
        pr = OrProblem()
        pr.N, pr.M, pr.kind, pr.n_groups = N, self.M, kind, G
        pr.group, pr.K, pr.S = p(self.group, C.c_int32), p(self.K, C.c_int32), p(self.S, C.c_double)
        pr.y, pr.bed = p(self.y, C.c_float), p(self.bed, C.c_uint8)
        pr.seed, pr.chain = seed, chain
        pr.v0E, pr.s02E, pr.v0G, pr.s02G = priors
        if perm_chain is not None:
            pr.shared_perm, pr.perm_chain = 1, perm_chain
        pr.dense_lut = 1 if dense_lut else 0
        pr.async_batch = int(async_batch)
        self.pr = pr
        h = C.c_void_p()
        rc = lib().or_markers_create(C.byref(pr), C.byref(h))
        if rc != 0:
            raise RuntimeError(f"oracle markers_create failed: {rc}")
        self.mk = h
        self.beta = np.zeros(self.M)
        self.comp = np.zeros(self.M, np.int32)
        self.acum = np.zeros(self.M)
        self.eps = np.zeros(N)
        st = OrState()
        st.beta, st.comp, st.acum, st.eps = (p(self.beta, C.c_double), p(self.comp, C.c_int32),
                                             p(self.acum, C.c_double), p(self.eps, C.c_double))
        self.st = st
        assert lib().or_init(C.byref(pr), C.byref(st)) == 0

    def __del__(self):
        try:
            lib().or_markers_destroy(self.mk)
        except Exception:
            pass

    def iterate(self, it):
        rc = lib().or_iterate(C.byref(self.pr), self.mk, C.byref(self.st), it)
        assert rc == 0, rc

    def sweep(self, order, u, z):
        o = np.ascontiguousarray(order, np.uint32)
        uu = np.ascontiguousarray(u, np.float64)
        zz = np.ascontiguousarray(z, np.float64)
        self.st.m0 = 0.0
        for i in range(OR_MAX_GROUPS * OR_MAX_K):
            self.st.v[i] = 0.0
        for i in range(OR_MAX_GROUPS):
            self.st.betasqnG[i] = 0.0
        lib().or_sweep(C.byref(self.pr), self.mk, C.byref(self.st), p(o, C.c_uint32), p(uu, C.c_double),
                       p(zz, C.c_double))

    def state(self):
        st = self.st
        return dict(beta=self.beta.copy(), comp=self.comp.copy(), acum=self.acum.copy(), eps=self.eps.copy(),
                    mu=st.mu, sigmaE=st.sigmaE, epsSum=st.epsSum, sigmaG=np.array(st.sigmaG[:self.G]),
                    pi=np.array(st.pi[:]).reshape(OR_MAX_GROUPS, OR_MAX_K)[:self.G].copy(),
                    v=np.array(st.v[:]).reshape(OR_MAX_GROUPS, OR_MAX_K)[:self.G].copy(),
                    betasqnG=np.array(st.betasqnG[:self.G]))

    def set_state(self, s):
        self.beta[:] = s["beta"]
        self.comp[:] = s["comp"]
        self.acum[:] = s["acum"]
        self.eps[:] = s["eps"]
        self.st.mu, self.st.sigmaE, self.st.epsSum = s["mu"], s["sigmaE"], s.get("epsSum", 0.0)
        for g in range(self.G):
            self.st.sigmaG[g] = s["sigmaG"][g]
            for k in range(OR_MAX_K):
                self.st.pi[g * OR_MAX_K + k] = s["pi"][g][k]
