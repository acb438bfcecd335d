"""PLINK file I/O and seeded synthetic genotype data.

File formats follow the reference readers: `.fam` (6 columns, src/data.cpp:85-107),
`.bim` (6 columns, src/data.cpp:109-133), SNP-major `.bed` with the magic
0x6c 0x1b 0x01 (src/preprocessgraph.cpp:195-200), phenotype file
`FID IID y` with rows whose value is "NA" skipped and the remaining values
packed in file order (src/data.cpp:334-365), and group file `SNP group`
(src/data.cpp:424-453).
"""
from __future__ import annotations

from pathlib import Path
from typing import Optional, Tuple

import numpy as np

BED_MAGIC = bytes([0x6C, 0x1B, 0x01])
# genotype (copies of allele 1) -> 2-bit code; missing -> 1
_G2CODE = np.array([3, 2, 0], dtype=np.uint8)


def encode_bed(g: np.ndarray) -> np.ndarray:
    """int8 genotypes (M x N; 0,1,2, -1 missing) -> BED payload (M x ceil(N/4))."""
    M, N = g.shape
    codes = np.where(g < 0, 1, _G2CODE[np.clip(g, 0, 2)]).astype(np.uint8)
    pad = (-N) % 4
    if pad:
        codes = np.concatenate([codes, np.zeros((M, pad), np.uint8)], axis=1)
    c = codes.reshape(M, -1, 4)
    return (c[:, :, 0] | (c[:, :, 1] << 2) | (c[:, :, 2] << 4) | (c[:, :, 3] << 6)).astype(np.uint8)


def decode_bed(payload: np.ndarray, N: int) -> np.ndarray:
    """BED payload (M x ceil(N/4)) -> int8 genotypes with -1 for missing."""
    M = payload.shape[0]
    b = payload.astype(np.uint8)
    codes = np.stack([(b >> (2 * k)) & 3 for k in range(4)], axis=2).reshape(M, -1)[:, :N]
    lut = np.array([2, -1, 1, 0], dtype=np.int8)
    return lut[codes]


def write_plink(prefix: str | Path, payload: np.ndarray, N: int, snp_ids=None, ind_ids=None):
    prefix = Path(prefix)
    M = payload.shape[0]
    with open(prefix.with_suffix(".bed"), "wb") as f:
        f.write(BED_MAGIC)
        f.write(np.ascontiguousarray(payload, np.uint8).tobytes())
    snp_ids = snp_ids or [f"snp{j + 1}" for j in range(M)]
    ind_ids = ind_ids or [f"ind{i + 1}" for i in range(N)]
    with open(prefix.with_suffix(".bim"), "w") as f:
        for j, s in enumerate(snp_ids):
            f.write(f"1\t{s}\t0\t{j + 1}\tA\tG\n")
    with open(prefix.with_suffix(".fam"), "w") as f:
        for i in ind_ids:
            f.write(f"{i} {i} 0 0 0 -9\n")


def read_fam(path: str | Path):
    ids = []
    with open(path) as f:
        for line in f:
            t = line.split()
            if len(t) >= 6:
                ids.append((t[0], t[1]))
    return ids


def read_bim(path: str | Path):
    ids = []
    with open(path) as f:
        for line in f:
            t = line.split()
            if len(t) >= 6:
                ids.append(t[1])
    return ids


def read_bed(path: str | Path, N: int, M: int) -> np.ndarray:
    raw = np.fromfile(path, dtype=np.uint8)
    if raw.size < 3 or bytes(raw[:3]) != BED_MAGIC:
        raise ValueError(f"{path}: incorrect first three bytes of bed file")
    cb = (N + 3) // 4
    if raw.size - 3 != M * cb:
        raise ValueError(f"{path}: problem with the BED file ... has the FAM/BIM file been changed?")
    return raw[3:].reshape(M, cb)


def write_phen(path: str | Path, y: np.ndarray, ind_ids=None):
    ind_ids = ind_ids or [f"ind{i + 1}" for i in range(len(y))]
    with open(path, "w") as f:
        for i, v in zip(ind_ids, y):
            f.write(f"{i} {i} {float(v)!r}\n")


def read_phen(path: str | Path, fam_ids) -> np.ndarray:
    """Values of known individuals in file order, "NA" skipped, as float32."""
    known = {f"{a}:{b}" for a, b in fam_ids}
    out = []
    with open(path) as f:
        for line in f:
            t = line.split()
            if len(t) >= 3 and f"{t[0]}:{t[1]}" in known and t[2] != "NA":
                out.append(float(t[2]))
    return np.array(out, dtype=np.float32)


def write_groups(path: str | Path, group: np.ndarray, snp_ids=None):
    snp_ids = snp_ids or [f"snp{j + 1}" for j in range(len(group))]
    with open(path, "w") as f:
        for s, g in zip(snp_ids, group):
            f.write(f"{s}\t{int(g)}\n")


def read_groups(path: str | Path) -> np.ndarray:
    g = []
    with open(path) as f:
        for line in f:
            t = line.split()
            if len(t) >= 2:
                g.append(int(t[1]))
    return np.array(g, dtype=np.int32)


# --------------------------------------------------------------------------
# Synthetic data (seeded).

def standardize_dense(g: np.ndarray) -> np.ndarray:
    """Dense standardisation of the reference (src/densemarkerbuilder.cpp:43-60), M x N float64."""
    x = g.astype(np.float64)
    miss = g < 0
    n = (~miss).sum(1)
    mean = np.where(miss, 0, x).sum(1) / n
    x = np.where(miss, mean[:, None], x)
    x -= x.mean(1, keepdims=True)
    x *= 1.0 / np.sqrt((x * x).sum(1) / (g.shape[1] - 1.0))[:, None]
    return x


def synth_genotypes(N: int, M: int, seed: int, p: Optional[np.ndarray] = None, missing: float = 0.0,
                    p_lo: float = 0.05, p_hi: float = 0.5) -> Tuple[np.ndarray, np.ndarray]:
    """g ~ Binomial(2, p_j) per marker, optional missing at random; no monomorphic markers."""
    rng = np.random.default_rng(seed)
    if p is None:
        p = rng.uniform(p_lo, p_hi, size=M)
    g = (rng.random((M, N)) < p[:, None]).astype(np.int8) + (rng.random((M, N)) < p[:, None]).astype(np.int8)
    # ensure every marker varies (the reference rejects markers that do not)
    for j in np.flatnonzero((g == g[:, :1]).all(1)):
        g[j, 0] = 1 if g[j, 0] != 1 else 0
    if missing > 0:
        m = rng.random((M, N)) < missing
        g[m] = -1
        for j in range(M):
            obs = g[j][g[j] >= 0]
            if obs.size < 2 or (obs == obs[0]).all():
                g[j, 0], g[j, 1] = 0, 1
    return g, p


def synth_phenotype(g: np.ndarray, seed: int, n_causal: int, h2: float) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """y = X b + e with X the standardised genotypes, b ~ N(0, h2/n_causal), e ~ N(0, 1-h2)."""
    rng = np.random.default_rng(seed + 7919)
    M, N = g.shape
    causal = np.sort(rng.choice(M, size=min(n_causal, M), replace=False))
    b = rng.normal(0.0, np.sqrt(h2 / len(causal)), size=len(causal))
    x = standardize_dense(g[causal])
    y = b @ x + rng.normal(0.0, np.sqrt(1.0 - h2), size=N)
    return y.astype(np.float32), causal, b
