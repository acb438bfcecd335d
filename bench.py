"""Benchmark of the GB300 BayesR Gibbs sweep (marker-updates per second).

Workload: dense 2-bit genotypes, N = 100,000 individuals x M = 100,000
markers, allele frequencies U(0.01, 0.5), two marker groups with separate
mixtures (S1 = 0.01,0.001,0.0001; S2 = 0.1,0.01), 1,000 causal markers with
beta ~ N(0, 0.4/1000), h2 = 0.4; seeded synthetic data generated on the device.
A step is one Gibbs iteration: updateMu, the per-marker draws, one sweep over
all M markers and the sigmaE / sigmaG / pi draws.  The chosen form (FP32
compensated residual with an FP64 refresh every 50 sweeps) is the headline;
the plain FP64 kernel is timed beside it on the same steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Beside the headline, the batching form is measured on its own workload
(64 chains with their own phenotypes on N = 50,000 x M = 200,000 shared
genotypes; the "batched" object): aggregate marker-updates/s of all chains
against the plain FP64 single-chain kernel on the same genotypes.

`--impl reference` times the reference algorithm's CPU implementation on the
host cores (the repository's FP64 restatement, since the reference itself
cannot be built: Eigen, Boost.Random and TBB are absent) on a bounded sample
of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_IND, M_SNP = 100_000, 100_000
DRAM_BYTES_PER_MARKER_N100K = 261.520286e9 * 1.287168e-3 / 8192
S_GROUPS = [[0.01, 0.001, 0.0001], [0.1, 0.01]]
P_LO, P_HI = 0.01, 0.5
N_CAUSAL, H2 = 1000, 0.4
SEED = 20261203
REFRESH = 50
PROFILE_STEPS = 2
METRIC = "marker-updates/sec at N=100k on 1 GB300, chosen vs plain FP64 GPU at matched beta error"
WORKLOAD = ("dense 2-bit BayesR, N=100,000 x M=100,000, two groups (S1=0.01,0.001,0.0001; S2=0.1,0.01), "
            "1,000 causal, h2=0.4")


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def peaks_bf16():
    """Dense bf16 tensor peak (TFLOP/s) for a kernel timed inside a long step:
    the sustained figure of MEASURED_PEAKS.json, else the fallback."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("bf16_tflops_sustained", d["bf16_tflops"]))
    return 1700.0


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            t = [x.strip() for x in line.split(",")]
            if len(t) < 9:
                continue
            try:
                sm.append(float(t[1]))
                smax = float(t[2])
            except ValueError:
                continue
            for nm, v in zip(names, t[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(gpus):
    rank, world = 0, 1
    if gpus > 1 or "RANK" in os.environ:
        import torch.distributed as dist
        rank = int(os.environ.get("RANK", 0))
        world = int(os.environ.get("WORLD_SIZE", gpus))
        dist.init_process_group("nccl" if os.environ.get("BRR_BENCH_GLOO") is None else "gloo")
        return rank, world, dist
    return rank, world, None


def max_over_ranks(x: float, dist, device=None) -> float:
    """The largest of every rank's x (one rank: x itself).  The tensor lives on
    the rank's GPU under NCCL and on the host under gloo."""
    if dist is None:
        return float(x)
    import torch
    on = "cpu" if dist.get_backend() == "gloo" else device
    t = torch.tensor([float(x)], dtype=torch.float64, device=on)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world: int, markers: int, steps: int, seconds: float) -> float:
    """Whole-job marker-updates/s of `world` replicas that each swept `markers`
    markers `steps` times, the slowest taking `seconds`."""
    return world * markers * steps / seconds


def make_problem(lib, gpu, torch, device, chain_id):
    """Synthetic BED payload on the device, phenotype from 1,000 causal markers."""
    cb = (N_IND + 3) // 4
    d_bed = torch.empty(M_SNP * cb, dtype=torch.uint8, device=device)
    gpu.synth_bed_device(d_bed.data_ptr(), N_IND, M_SNP, SEED, P_LO, P_HI, 0.0, lib=lib)
    rng = np.random.default_rng(SEED)
    causal = np.sort(rng.choice(M_SNP, N_CAUSAL, replace=False)).astype(np.uint32)
    b = rng.normal(0.0, np.sqrt(H2 / N_CAUSAL), N_CAUSAL)
    group = (np.arange(M_SNP) >= M_SNP // 2).astype(np.int32)
    probe = gpu.Chain(gpu.ChainConfig(N=N_IND, M=M_SNP, S=S_GROUPS, device=device), lib=lib)
    probe.pack_bed_device(d_bed.data_ptr(), d_bed.numel())
    gv = probe.xbeta(causal, b)
    probe.close()
    y = (gv + rng.normal(0.0, np.sqrt(1.0 - H2), N_IND)).astype(np.float32)
    return d_bed, y, group


def run_form(lib, gpu, torch, device, d_bed, y, group, form, steps, warmup, chain_id, barrier, profile=False):
    """Warm-up iterations, then exactly `steps` timed iterations between two
    barriers (device synchronised on every rank); the time reported is the
    library's CUDA-event time of those iterations."""
    cfg = gpu.ChainConfig(N=N_IND, M=M_SNP, S=S_GROUPS, form=form, seed=SEED + chain_id, chain=chain_id,
                          refresh_every=REFRESH if form == gpu.FORM_FP32C else 0, device=device)
    ch = gpu.Chain(cfg, lib=lib)
    ch.pack_bed_device(d_bed.data_ptr(), d_bed.numel())
    ch.set_groups(group)
    ch.set_phenotype(y)
    ch.init()
    gram = ch.gram_info()
    ch.iterate(warmup)
    barrier()
    t0 = time.perf_counter()
    ch.iterate(steps)
    barrier()
    wall = time.perf_counter() - t0
    sweep_ms, total_ms, rounds = ch.timing()
    st = ch.state()
    # phase counters from PROFILE_STEPS further iterations of the counting
    # variant, after the timed steps and the state read
    phases = np.zeros(16, np.int64)
    if profile:
        ch.set_profiling(True)
        ch.iterate(PROFILE_STEPS)
        phases = ch.phase_cycles()
    ch.close()
    return dict(total_ms=total_ms, sweep_ms=sweep_ms, rounds=rounds, wall_s=wall, phases=phases.tolist(),
                beta=st["beta"], comp=st["comp"], sigmaE=st["sigmaE"], sigmaG=st["sigmaG"].tolist(), gram=gram)


def run_e2e(lib, gpu, torch, device, host_bed, y, group, steps, chain_id):
    """The same chain through the C ABI from host buffers: BED upload from
    pinned memory and device packing inside the timed region, and every step
    reads the sample row (beta, comp, acum, residual) back to the host, as the
    reference's sample writer consumes it."""
    cfg = gpu.ChainConfig(N=N_IND, M=M_SNP, S=S_GROUPS, form=gpu.FORM_FP32C, seed=SEED + chain_id,
                          chain=chain_id, refresh_every=REFRESH, device=device)
    ch = gpu.Chain(cfg, lib=lib)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    ch.pack_bed(host_bed)
    ch.set_groups(group)
    ch.set_phenotype(y)
    t1 = time.perf_counter()
    ch.init()
    t2 = time.perf_counter()
    d2h = 0
    for _ in range(steps):
        ch.iterate(1)
        st = ch.state()
        d2h += st["beta"].nbytes + st["comp"].nbytes + st["acum"].nbytes + st["eps"].nbytes
    torch.cuda.synchronize(device)
    wall = time.perf_counter() - t0
    gram_ms = ch.gram_info()["build_ms"]
    ch.close()
    h2d = host_bed.nbytes + y.nbytes + group.nbytes
    # where the end-to-end time goes (host clock): upload and packing, the
    # chain's set-up (marker Gram: allocation and device build), the iterations
    # with their read-backs
    parts = {"upload_and_pack_s": t1 - t0, "init_s": t2 - t1, "gram_build_device_s": gram_ms / 1e3,
             "iterations_s": wall - (t2 - t0)}
    return dict(wall=wall, h2d_per_step=h2d / steps, d2h_per_step=d2h / steps, parts=parts)


# Batching form: 64 chains (distinct seeds, one phenotype each) on shared
# genotypes, N = 50,000 x M = 200,000, p ~ U(0.01, 0.5), 1,000 causal markers per
# phenotype with h2 ~ U(0.1, 0.7); marker blocks of 32 on the tensor cores.
B_N, B_M, B_C = 50_000, 200_000, 64
B_WORKLOAD = ("batched BayesR, 64 chains (distinct seeds, 64 phenotypes h2~U(0.1,0.7), 1,000 causal each) on shared "
              "dense genotypes N=50,000 x M=200,000, p~U(0.01,0.5), blocks of 32, S=0.01,0.001,0.0001")


def run_batched(lib, gpu, torch, device, steps, warmup):
    """Aggregate marker-updates/s of the 64-chain tensor-core form and of the
    plain FP64 single-chain kernel on the same genotypes."""
    S = [[0.01, 0.001, 0.0001]]
    seed = SEED + 7
    cb = (B_N + 3) // 4
    d_bed = torch.empty(B_M * cb, dtype=torch.uint8, device=device)
    gpu.synth_bed_device(d_bed.data_ptr(), B_N, B_M, seed, P_LO, P_HI, 0.0, lib=lib)
    probe = gpu.Chain(gpu.ChainConfig(N=B_N, M=B_M, S=S, device=device), lib=lib)
    probe.pack_bed_device(d_bed.data_ptr(), d_bed.numel())
    rng = np.random.default_rng(seed)
    ys = np.zeros((B_C, B_N), np.float32)
    for c in range(B_C):
        h2 = rng.uniform(0.1, 0.7)
        causal = np.sort(rng.choice(B_M, N_CAUSAL, replace=False)).astype(np.uint32)
        b = rng.normal(0.0, np.sqrt(h2 / N_CAUSAL), N_CAUSAL)
        ys[c] = probe.xbeta(causal, b) + rng.normal(0.0, np.sqrt(1.0 - h2), B_N)
    probe.close()
    bt = gpu.Batch(gpu.ChainConfig(N=B_N, M=B_M, S=S, seed=seed, device=device), B_C, lib=lib)
    bt.pack_bed_device(d_bed.data_ptr(), d_bed.numel())
    bt.set_phenotypes(ys)
    bt.init()
    geo = bt.geometry()
    bt.iterate(warmup)
    torch.cuda.synchronize(device)
    bt.iterate(steps)
    torch.cuda.synchronize(device)
    b_sweep, b_total, _ = bt.timing()
    # phase counters from one further iteration of the counting kernel variant
    bt.set_profiling(True)
    bt.iterate(1)
    cyc = bt.timing()[2]
    bt.close()
    ch = gpu.Chain(gpu.ChainConfig(N=B_N, M=B_M, S=S, seed=seed, form=gpu.FORM_FP64, device=device), lib=lib)
    ch.pack_bed_device(d_bed.data_ptr(), d_bed.numel())
    ch.set_phenotype(ys[0])
    ch.init()
    p_steps = 2
    ch.iterate(1)
    ch.iterate(p_steps)
    p_sweep, p_total, _ = ch.timing()
    ch.close()
    del d_bed
    torch.cuda.empty_cache()
    nblocks = (B_M + 31) // 32
    # algorithmic tensor work per block: X_block^T E and X_block dB (2 * 32 * C * N
    # each) plus the block Gram (32 * 32 * N); the kernel computes the residual
    # as four 11-bit limbs, i.e. four times the dot and update products
    alg_flop = nblocks * (2 * 2 * 32 * B_C * B_N + 2 * 32 * 32 * B_N)
    issued_flop = nblocks * (2 * 2 * 32 * 4 * B_C * B_N + 2 * 128 * 32 * B_N)
    sweep_s = b_sweep / 1e3 / steps
    rate = B_C * B_M * steps / (b_total / 1e3)
    plain = B_M * p_steps / (p_total / 1e3)
    return dict(rate=rate, total_s=b_total / 1e3, ms_per_step=b_total / steps, sweep_ms=b_sweep / steps,
                plain=plain,
                plain_ms=p_total / p_steps, alg_tflops=alg_flop / sweep_s / 1e12,
                issued_tflops=issued_flop / sweep_s / 1e12,
                cycles=(cyc / nblocks).tolist(), geometry=geo)


# Uneven batch: 32 independent regressions of different sizes in one launch per
# iteration; N log-uniform in [1,000, 200,000], M log-uniform in [5,000, 500,000],
# allele frequencies Beta(0.5, 2) clipped to [0.001, 0.5], 1 % missing, h2 ~ U(0.2, 0.6),
# 0.5 % causal markers; the FP32C restart form with the FP64 refresh every 50 sweeps.
U_N = (1_000, 200_000)
U_M = (5_000, 500_000)
U_WORKLOAD = ("uneven batch of 32 regressions in one launch per iteration: N log-U[1k, 200k], M log-U[5k, 500k], "
              "p~Beta(0.5,2) clipped [0.001,0.5], 1% missing, h2~U(0.2,0.6), 0.5% causal, dense or ragged per "
              "instance, FP32C restart form, S=0.01,0.001,0.0001")


def uneven_instances(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    n = 32
    N = np.exp(rng.uniform(np.log(U_N[0]), np.log(U_N[1]), n)) * scale
    M = np.exp(rng.uniform(np.log(U_M[0]), np.log(U_M[1]), n)) * scale
    N = np.maximum(N.astype(np.int64), 256)
    M = np.maximum(M.astype(np.int64), 200)
    h2 = rng.uniform(0.2, 0.6, n)
    return N, M, h2


def run_uneven(lib, gpu, torch, device, steps, tune_rounds, scale=1.0):
    """Aggregate marker-updates/s of 32 regressions of different sizes swept
    together (one cooperative launch per iteration, CTAs and round widths from
    the autotuner)."""
    S = [[0.01, 0.001, 0.0001]]
    seed = SEED + 11
    N, M, h2 = uneven_instances(seed, scale)
    # each instance's genotypes and phenotype; its kind, dense or ragged, from
    # its own packed genotype counts: the ragged sweep reads 2 bytes (a
    # slice-local index) per listed genotype (ones, twos, missing), the dense
    # sweep N/4 bytes per marker, so ragged storage is chosen when fewer than one
    # genotype in eight is listed
    rng = np.random.default_rng(seed + 2)
    beds, ys, kinds, listed = [], [], [], []
    for i in range(len(N)):
        n_i, m_i = int(N[i]), int(M[i])
        d_bed = torch.empty(m_i * ((n_i + 3) // 4), dtype=torch.uint8, device=device)
        gpu.synth_bed_device_beta(d_bed.data_ptr(), n_i, m_i, seed + i, 0.5, 2.0, 0.001, 0.5, 0.01, lib=lib)
        probe = gpu.Chain(gpu.ChainConfig(N=n_i, M=m_i, S=S, device=device), lib=lib)
        probe.pack_bed_device(d_bed.data_ptr(), d_bed.numel())
        n_c = max(1, int(0.005 * m_i))
        causal = np.sort(rng.choice(m_i, n_c, replace=False)).astype(np.uint32)
        b = rng.normal(0.0, np.sqrt(h2[i] / n_c), n_c)
        ys.append((probe.xbeta(causal, b) + rng.normal(0.0, np.sqrt(1.0 - h2[i]), n_i)).astype(np.float32))
        _, counts = probe.marker_table()
        probe.close()
        frac = float(counts[:, 1:4].sum()) / (float(n_i) * float(m_i))
        listed.append(frac)
        kinds.append(gpu.KIND_RAGGED if 2.0 * frac < 0.25 else gpu.KIND_DENSE)
        beds.append(d_bed)
    cfgs = [gpu.ChainConfig(N=int(N[i]), M=int(M[i]), kind=kinds[i], form=gpu.FORM_FP32C, S=S, seed=seed,
                            chain=i, refresh_every=REFRESH, device=device) for i in range(len(N))]
    mm = gpu.Multi(cfgs, lib=lib)
    for i in range(len(N)):
        mm.pack_bed_device(i, beds[i].data_ptr(), beds[i].numel())
        mm.set_phenotype(i, ys[i])
    del beds
    torch.cuda.empty_cache()
    mm.init()
    t0 = mm.timing()
    mm.tune(tune_rounds)
    tuned = mm.timing()
    mm.iterate(steps)
    t = mm.timing()
    mm.close()
    total_m = int(M.sum())
    inst = t["inst_ms"]
    return dict(rate=total_m * steps / (t["total_ms"] / 1e3), total_s=t["total_ms"] / 1e3,
                ms_per_step=t["total_ms"] / steps,
                sweep_ms=t["sweep_ms"] / steps, instances=len(N), total_markers=total_m,
                total_genotypes=float((N.astype(float) * M.astype(float)).sum()),
                kinds={"dense": kinds.count(gpu.KIND_DENSE), "ragged": kinds.count(gpu.KIND_RAGGED),
                       "rule": "ragged when fewer than 1 in 8 genotypes are listed (2-byte indices vs N/4 "
                               "bytes per marker), from each instance's packed counts",
                       "listed_fraction_min_max": [round(min(listed), 4), round(max(listed), 4)]},
                ctas_first=t0["ctas"].tolist(), ctas=t["ctas"].tolist(), widths=t["width"].tolist(),
                inst_ms=[round(x, 3) for x in inst.tolist()],
                balance_max_over_mean=float(inst.max() / max(inst.mean(), 1e-9)),
                N=N.tolist(), M=M.tolist())


# Ragged sparse markers (the C2 configuration): N = 20,000 x M = 50,000, 70 % of
# the markers rare (p ~ U(0.001, 0.05)), the rest p ~ U(0.05, 0.5), 1 % missing
# genotypes, 500 causal markers with beta ~ N(0, 0.5/500), h2 = 0.5; the plain
# FP64 form against the FP32C form with the FP64 refresh every 50 sweeps.
R_N, R_M, R_RARE = 20_000, 50_000, 35_000
R_LATE = 190   # untimed iterations between the burn-in and the stationary timing
R_WORKLOAD = ("ragged sparse BayesR, N=20,000 x M=50,000, 70% rare p~U(0.001,0.05), rest p~U(0.05,0.5), 1% missing, "
              "500 causal, h2=0.5, S=0.01,0.001,0.0001")
# The plain dense configuration C1 (CPU-runnable): N = 2,000 x M = 5,000,
# p ~ U(0.05, 0.5), 100 causal, h2 = 0.5.
C1_N, C1_M = 2_000, 5_000
S1 = [[0.01, 0.001, 0.0001]]


def synth_parts(torch, gpu, lib, device, N, parts, seed, missing):
    """Concatenated device BED payloads, one per (markers, p_lo, p_hi) part."""
    cb = (N + 3) // 4
    out = []
    for k, (m, lo, hi) in enumerate(parts):
        d = torch.empty(m * cb, dtype=torch.uint8, device=device)
        gpu.synth_bed_device(d.data_ptr(), N, m, seed + k, lo, hi, missing, lib=lib)
        out.append(d)
    return torch.cat(out) if len(out) > 1 else out[0]


def synth_phenotype(gpu, lib, device, d_bed, N, M, n_causal, h2, seed):
    """Phenotype from n_causal standardised columns (effects N(0, h2/n_causal))
    plus N(0, 1-h2) noise, and the markers' genotype counts."""
    rng = np.random.default_rng(seed)
    probe = gpu.Chain(gpu.ChainConfig(N=N, M=M, S=S1, device=device), lib=lib)
    probe.pack_bed_device(d_bed.data_ptr(), d_bed.numel())
    causal = np.sort(rng.choice(M, n_causal, replace=False)).astype(np.uint32)
    b = rng.normal(0.0, np.sqrt(h2 / n_causal), n_causal)
    y = (probe.xbeta(causal, b) + rng.normal(0.0, np.sqrt(1.0 - h2), N)).astype(np.float32)
    _, counts = probe.marker_table()
    probe.close()
    return y, counts


def time_chain(gpu, lib, device, d_bed, N, M, y, kind, form, steps, warmup, seed, gram=0, late=0, phases=False,
               pair_rounds=0):
    """W warm-up and K timed iterations of one chain; the library's CUDA-event
    time of the timed ones.  late > 0: then `late` more untimed iterations and
    K timed again (the chain's stationary phase)."""
    ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=kind, form=form, S=S1, seed=seed, gram=gram, pair_rounds=pair_rounds,
                                   refresh_every=REFRESH if form == gpu.FORM_FP32C else 0, device=device), lib=lib)
    ch.pack_bed_device(d_bed.data_ptr(), d_bed.numel())
    ch.set_phenotype(y)
    ch.init()
    ch.iterate(warmup)
    ch.iterate(steps)
    sweep_ms, total_ms, rounds = ch.timing()
    st = ch.state()
    out = dict(rate=M * steps / (total_ms / 1e3), ms_per_step=total_ms / steps, sweep_ms=sweep_ms / steps,
               rounds=rounds / steps, beta=st["beta"], comp=st["comp"], sigmaE=st["sigmaE"])
    if phases:
        # one further iteration of the phase-counting variant: cycles per round on CTA 0
        ch.set_profiling(1)
        ch.iterate(1)
        ph = ch.phase_cycles()
        ch.set_profiling(0)
        n = max(int(ph[5]), 1)
        names = ("ring", "dot_products", "exchange_wait", "sampling", "update")
        out["phase_cycles_per_round"] = {k: round(float(ph[i]) / n) for i, k in enumerate(names)}
        if ph[6] or ph[7]:
            out["phase_cycles_per_round"]["dot_products"] = round(float(ph[6]) / n)
            out["phase_cycles_per_round"]["pair_terms"] = round(float(ph[7]) / n)
            out["phase_cycles_per_round"]["publication"] = round(float(ph[1]) / n)
        out["phase_iteration"] = warmup + steps + 1
        warmup += 1
    if late:
        ch.iterate(late)
        ch.iterate(steps)
        _, lt, lr = ch.timing()
        out["late"] = {"after_iterations": warmup + steps + late, "rate": M * steps / (lt / 1e3),
                       "ms_per_step": lt / steps, "rounds_per_step": lr / steps,
                       "nonzero_effects": int(np.count_nonzero(ch.state()["beta"]))}
    ch.close()
    return out



def cpu_rate(bed, N, y, kind, iters):
    """Rate of the FP64 restatement (fast-flags build, one core) over all
    markers of a small configuration, after one untimed iteration."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as O
    O.use_timing_build()
    oc = O.OracleChain(np.ascontiguousarray(bed), N, y, S1, kind=kind, seed=SEED)
    oc.iterate(0)
    t0 = time.perf_counter()
    for it in range(1, 1 + iters):
        oc.iterate(it)
    dt = time.perf_counter() - t0
    return {"value": bed.shape[0] * iters / dt, "unit": "marker-updates/s", "cores": 1, "kind": "port",
            "sample": f"all {bed.shape[0]} markers x N={N}, {iters} Gibbs iterations after one untimed ({dt:.1f} s), "
                      f"FP64 restatement built -O3 -ffast-math -funroll-loops"}


def run_ragged(lib, gpu, torch, device, steps, warmup, cpu=True):
    """C2: the FP64 and FP32C ragged chains, their rates and the roofline on
    the index bytes; C1: the plain FP64 dense chain; the CPU restatement's
    rate on both beside them."""
    d_bed = synth_parts(torch, gpu, lib, device, R_N, [(R_RARE, 0.001, 0.05), (R_M - R_RARE, 0.05, 0.5)], SEED + 21,
                        0.01)
    y, counts = synth_phenotype(gpu, lib, device, d_bed, R_N, R_M, 500, 0.5, SEED + 21)
    f64 = time_chain(gpu, lib, device, d_bed, R_N, R_M, y, gpu.KIND_RAGGED, gpu.FORM_FP64, steps, warmup, SEED)
    # the first timed iterations lie in the chain's burn-in, where about one
    # marker in six changes its effect; the late ones in its stationary phase
    f32 = time_chain(gpu, lib, device, d_bed, R_N, R_M, y, gpu.KIND_RAGGED, gpu.FORM_FP32C, steps, warmup, SEED,
                     late=R_LATE, phases=True)
    f32r = time_chain(gpu, lib, device, d_bed, R_N, R_M, y, gpu.KIND_RAGGED, gpu.FORM_FP32C, steps, warmup, SEED,
                      pair_rounds=-1, late=R_LATE)
    # algorithmic bytes of a sweep: 4 bytes per listed genotype (ones, twos, missing)
    idx_bytes = 4.0 * float(counts[:, 1:4].sum())
    hbm, _ = peaks()
    achieved = idx_bytes / (f32["sweep_ms"] / 1e3) / 1e9
    host_bed = d_bed.cpu().numpy().reshape(R_M, -1)
    del d_bed
    c1_bed = synth_parts(torch, gpu, lib, device, C1_N, [(C1_M, 0.05, 0.5)], SEED + 31, 0.0)
    c1_y, _ = synth_phenotype(gpu, lib, device, c1_bed, C1_N, C1_M, 100, 0.5, SEED + 31)
    c1 = time_chain(gpu, lib, device, c1_bed, C1_N, C1_M, c1_y, gpu.KIND_DENSE, gpu.FORM_FP64, 10, 3, SEED)
    c1c = time_chain(gpu, lib, device, c1_bed, C1_N, C1_M, c1_y, gpu.KIND_DENSE, gpu.FORM_FP32C, 10, 3, SEED)
    c1_host = c1_bed.cpu().numpy().reshape(C1_M, -1)
    del c1_bed
    torch.cuda.empty_cache()
    out = {
        "workload": R_WORKLOAD, "value": f32["rate"], "unit": "marker-updates/s",
        "form": "fp32c (refresh 50); pair-resolved rounds of 32 markers while more than M/40 effects are non-zero, "
                "restart rounds otherwise",
        "timed_iterations": f"{warmup + 1}..{warmup + steps} (burn-in)",
        "steps": steps, "ms_per_step": f32["ms_per_step"], "sweep_ms": f32["sweep_ms"], "rounds_per_step": f32["rounds"],
        "stationary": f32["late"],
        "phase_cycles_per_round": f32["phase_cycles_per_round"], "phase_iteration": f32["phase_iteration"],
        "fp32c_restart_rounds": {"value": f32r["rate"], "ms_per_step": f32r["ms_per_step"],
                                 "rounds_per_step": f32r["rounds"], "stationary": f32r["late"],
                                 "component_mismatches_vs_pair_rounds": int(np.count_nonzero(f32r["comp"] != f32["comp"]))},
        "plain_fp64": {"value": f64["rate"], "ms_per_step": f64["ms_per_step"], "rounds_per_step": f64["rounds"]},
        "speedup_fp32c_vs_plain": f32["rate"] / f64["rate"],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": None, "kernel": "k_sweep_pr (ragged, FP32C, pair-resolved rounds)",
                     "algorithmic_bytes_per_launch": idx_bytes,
                     "note": "4 bytes per listed genotype (ones, twos, missing) per sweep"},
        "matched_error": {"beta_max_abs_diff_vs_plain": float(np.abs(f32["beta"] - f64["beta"]).max()),
                          "component_mismatches_vs_plain": int(np.count_nonzero(f32["comp"] != f64["comp"])),
                          "sigmaE_rel_diff_vs_plain": abs(f32["sigmaE"] / f64["sigmaE"] - 1),
                          "compared": "final state after the warm-up and timed iterations (same draws)"},
        "c1_dense_fp64": {"workload": "plain dense BayesR, N=2,000 x M=5,000, p~U(0.05,0.5), 100 causal, h2=0.5",
                          "value": c1["rate"], "ms_per_step": c1["ms_per_step"], "unit": "marker-updates/s",
                          "fp32c_gram_blocked": {"value": c1c["rate"], "ms_per_step": c1c["ms_per_step"]}},
    }
    if cpu:
        out["cpu_baseline"] = cpu_rate(host_bed, R_N, y, 1, 3)
        out["c1_dense_fp64"]["cpu_baseline"] = cpu_rate(c1_host, C1_N, c1_y, 0, 10)
    return out


def posterior_pair(a, b, n_iter, burn, thin, G, kmax):
    """Two chains on the same draws, iterated in lockstep: posterior means of
    beta, sigmaG and sigmaE and per-marker component frequencies over the kept
    iterations (after `burn`, every `thin`-th), and the iterations whose
    components differ between the two chains."""
    sums = [None, None]
    n_kept = 0
    mismatch_iters, mismatches, first = 0, 0, None
    t = [0.0, 0.0]
    for it in range(n_iter):
        for k, ch in enumerate((a, b)):
            t0 = time.perf_counter()
            ch.iterate(1)
            t[k] += time.perf_counter() - t0
        sa, sb = a.state(), b.state()
        d = int(np.count_nonzero(sa["comp"] != sb["comp"]))
        if d:
            mismatch_iters += 1
            mismatches += d
            first = it if first is None else first
        if it >= burn and (it - burn) % thin == 0:
            n_kept += 1
            for k, s in enumerate((sa, sb)):
                freq = np.zeros((s["comp"].size, kmax))
                freq[np.arange(s["comp"].size), s["comp"]] = 1.0
                cur = dict(beta=s["beta"], sigmaG=np.asarray(s["sigmaG"], float), sigmaE=s["sigmaE"], freq=freq)
                if sums[k] is None:
                    sums[k] = {kk: np.array(v, dtype=float, copy=True) for kk, v in cur.items()}
                else:
                    for kk, v in cur.items():
                        sums[k][kk] += v
    ma = {k: v / n_kept for k, v in sums[0].items()}
    mb = {k: v / n_kept for k, v in sums[1].items()}
    nz = mb["beta"] != 0
    floor = 1e-6 * float(np.abs(mb["beta"]).max())
    rel_beta = np.abs(ma["beta"] - mb["beta"])[nz] / np.maximum(np.abs(mb["beta"][nz]), floor)
    return {
        "iterations": n_iter, "burn_in": burn, "thin": thin, "kept": n_kept,
        "posterior_mean_beta_max_rel_diff": float(rel_beta.max()) if rel_beta.size else 0.0,
        "posterior_mean_beta_rel_floor": floor,
        "posterior_mean_beta_max_abs_diff": float(np.abs(ma["beta"] - mb["beta"]).max()),
        "posterior_mean_sigmaG_max_rel_diff": float(np.max(np.abs(ma["sigmaG"] / mb["sigmaG"] - 1))),
        "posterior_mean_sigmaE_rel_diff": float(abs(ma["sigmaE"] / mb["sigmaE"] - 1)),
        "component_frequency_max_abs_diff": float(np.abs(ma["freq"] - mb["freq"]).max()),
        "iterations_with_component_mismatch": mismatch_iters, "component_mismatches": mismatches,
        "first_mismatch_iteration": first,
        "markers_with_nonzero_posterior_mean_beta": int(nz.sum()),
        "posterior_mean_sigmaG_plain": mb["sigmaG"].tolist(), "posterior_mean_sigmaE_plain": float(mb["sigmaE"]),
        "wall_s_chosen": t[0], "wall_s_plain": t[1],
    }


def run_matched_chains(lib, gpu, torch, device, c3_iters, c2_iters):
    """The chosen forms against the plain FP64 chain (itself within 1e-10 of
    the FP64 oracle per iteration) over whole chains on the same draws: C3
    (1,000 iterations, burn-in 200) and C2 (2,000 iterations, burn-in 500,
    thin 5)."""
    out = {}
    d_bed, y, group = make_problem(lib, gpu, torch, device, 0)
    mk = []
    for form in (gpu.FORM_FP32C, gpu.FORM_FP64):
        cfg = gpu.ChainConfig(N=N_IND, M=M_SNP, S=S_GROUPS, form=form, seed=SEED, chain=0,
                              refresh_every=REFRESH if form == gpu.FORM_FP32C else 0, device=device)
        ch = gpu.Chain(cfg, lib=lib)
        ch.pack_bed_device(d_bed.data_ptr(), d_bed.numel())
        ch.set_groups(group)
        ch.set_phenotype(y)
        ch.init()
        mk.append(ch)
    out["c3"] = {"workload": WORKLOAD, "chosen": "fp32c gram-blocked" if mk[0].gram_info()["blocked"] else "fp32c",
                 **posterior_pair(mk[0], mk[1], c3_iters, min(200, c3_iters // 5), 1, 2, 4)}
    for ch in mk:
        ch.close()
    del d_bed
    torch.cuda.empty_cache()
    d_bed = synth_parts(torch, gpu, lib, device, R_N, [(R_RARE, 0.001, 0.05), (R_M - R_RARE, 0.05, 0.5)], SEED + 21,
                        0.01)
    y, _ = synth_phenotype(gpu, lib, device, d_bed, R_N, R_M, 500, 0.5, SEED + 21)
    mk = []
    for form in (gpu.FORM_FP32C, gpu.FORM_FP64):
        ch = gpu.Chain(gpu.ChainConfig(N=R_N, M=R_M, kind=gpu.KIND_RAGGED, form=form, S=S1, seed=SEED,
                                       refresh_every=REFRESH if form == gpu.FORM_FP32C else 0, device=device), lib=lib)
        ch.pack_bed_device(d_bed.data_ptr(), d_bed.numel())
        ch.set_phenotype(y)
        ch.init()
        mk.append(ch)
    out["c2"] = {"workload": R_WORKLOAD, "chosen": "fp32c (refresh 50)",
                 **posterior_pair(mk[0], mk[1], c2_iters, min(500, c2_iters // 4), 5, 1, 4)}
    for ch in mk:
        ch.close()
    return out


def run_cluster_compare(lib, gpu, torch, device, steps, warmup):
    """The restart sweep with its partial sums exchanged through L2 and a
    grid-wide barrier (one CTA per 64-individual chunk up to one per SM)
    against the same sweep as one thread-block cluster of 16, 8 or 4 CTAs
    (exchange through distributed shared memory): C1 dense and C2 ragged, FP64
    and FP32C forms, per-iteration time and the per-round phase cycles of
    CTA 0 (one further iteration of the counting variant); C3 dense FP32C for
    two iterations (grid-wide restart sweep against a cluster of 16)."""
    def one(d_bed, N, M, y, kind, form, cluster, group=None, S=S1, n_steps=steps, n_warm=warmup, spec=0):
        ch = gpu.Chain(gpu.ChainConfig(N=N, M=M, kind=kind, form=form, S=S, seed=SEED, device=device, gram=-1,
                                       pair_rounds=-1, spec_width=spec,
                                       refresh_every=REFRESH if form == gpu.FORM_FP32C else 0, cluster=cluster),
                       lib=lib)
        ch.pack_bed_device(d_bed.data_ptr(), d_bed.numel())
        if group is not None:
            ch.set_groups(group)
        ch.set_phenotype(y)
        ch.init()
        ch.iterate(n_warm)
        ch.iterate(n_steps)
        _, tot, rounds = ch.timing()
        ch.set_profiling(1)
        ch.iterate(1)
        ph = ch.phase_cycles()
        ch.close()
        r = max(int(ph[5]), 1)
        names = ("ring", "dot_products", "exchange_wait", "sampling", "update")
        return {"ms_per_step": tot / n_steps, "rate": M * n_steps / (tot / 1e3), "rounds_per_step": rounds / n_steps,
                "cycles_per_round": {k: round(float(ph[i]) / r) for i, k in enumerate(names)}}

    out = {}
    c1 = synth_parts(torch, gpu, lib, device, C1_N, [(C1_M, 0.05, 0.5)], SEED + 31, 0.0)
    c1_y, _ = synth_phenotype(gpu, lib, device, c1, C1_N, C1_M, 100, 0.5, SEED + 31)
    for form, fname in ((gpu.FORM_FP64, "fp64"), (gpu.FORM_FP32C, "fp32c_restart")):
        out[f"c1_dense_{fname}"] = {f"cluster_{cl}" if cl else "grid": one(c1, C1_N, C1_M, c1_y, gpu.KIND_DENSE, form, cl)
                                    for cl in (0, 16, 8, 4)}
    del c1
    d_bed = synth_parts(torch, gpu, lib, device, R_N, [(R_RARE, 0.001, 0.05), (R_M - R_RARE, 0.05, 0.5)], SEED + 21,
                        0.01)
    y, _ = synth_phenotype(gpu, lib, device, d_bed, R_N, R_M, 500, 0.5, SEED + 21)
    for form, fname in ((gpu.FORM_FP64, "fp64"), (gpu.FORM_FP32C, "fp32c")):
        out[f"c2_ragged_{fname}"] = {f"cluster_{cl}" if cl else "grid": one(d_bed, R_N, R_M, y, gpu.KIND_RAGGED, form,
                                                                             cl) for cl in (0, 16, 8, 4)}
    del d_bed
    torch.cuda.empty_cache()
    d_bed, y, group = make_problem(lib, gpu, torch, device, 0)
    # a cluster CTA holds 6,250 individuals: 16 markers per round keep its
    # ring of code slices and its residual slice within shared memory
    out["c3_dense_fp32c_restart"] = {f"cluster_{cl}" if cl else "grid": one(d_bed, N_IND, M_SNP, y, gpu.KIND_DENSE,
                                                                            gpu.FORM_FP32C, cl, group=group,
                                                                            S=S_GROUPS, n_steps=2, n_warm=1,
                                                                            spec=16 if cl else 0)
                                     for cl in (0, 16)}
    del d_bed
    torch.cuda.empty_cache()
    out["workloads"] = {"c1": "dense, N=2,000 x M=5,000, p~U(0.05,0.5), 100 causal, h2=0.5", "c2": R_WORKLOAD,
                        "c3": WORKLOAD}
    return out


def run_sample_writer(lib, gpu, torch, device, iters):
    """brr ppbayes on the benchmark workload (N = M = 100,000, two groups,
    FP32C form) from PLINK files: the mean iteration time with no sample
    rows, with a row every 5th iteration (thin 5, the C3 chain's setting) and
    with a row every iteration; a row holds 3M + N + 4 numbers."""
    import re
    import tempfile
    from bayesrrcmd_gb300 import plink
    from bayesrrcmd_gb300.build import build_cli
    cli = build_cli()
    d_bed, y, group = make_problem(lib, gpu, torch, device, 0)
    payload = d_bed.cpu().numpy().reshape(M_SNP, -1)
    del d_bed
    torch.cuda.empty_cache()
    out = {"workload": WORKLOAD + ", brr --form fp32c from PLINK files", "iterations": iters}
    with tempfile.TemporaryDirectory(dir=os.environ.get("BRR_SCRATCH")) as td:
        prefix = Path(td) / "c3"
        plink.write_plink(prefix, payload, N_IND)
        plink.write_phen(Path(td) / "c3.phen", y)
        plink.write_groups(Path(td) / "c3.group", group)
        del payload
        for name, burn, thin in (("no_rows", iters, 1), ("thin5", 0, 5), ("thin1", 0, 1)):
            samples = Path(td) / f"{name}.csv"
            cmd = [str(cli), "--analysis-type", "ppbayes", "--bfile", str(prefix), "--pheno", str(Path(td) / "c3.phen"),
                   "--group", str(Path(td) / "c3.group"), "--S", "0.01,0.001,0.0001;0.1,0.01", "--form", "fp32c",
                   "--chain-length", str(iters), "--burn-in", str(burn), "--thin", str(thin),
                   "--mcmc-samples", str(samples), "--seed", str(SEED)]
            t0 = time.perf_counter()
            r = subprocess.run(cmd, capture_output=True, text=True)
            wall = time.perf_counter() - t0
            if r.returncode != 0:
                raise RuntimeError(f"brr failed: {r.stderr[-2000:]}")
            it_s = float(re.search(r"mean iteration duration: ([0-9.eE+-]+)s", r.stdout).group(1))
            sw_s = float(re.search(r"mean flowgraph duration: ([0-9.eE+-]+)s", r.stdout).group(1))
            rows = max(0, sum(1 for _ in open(samples)) - 1) if samples.exists() else 0
            out[name] = {"mean_iteration_ms": 1e3 * it_s, "mean_sweep_ms": 1e3 * sw_s, "rows": rows,
                         "sample_file_bytes": samples.stat().st_size if samples.exists() else 0,
                         "wall_s": wall}
            if samples.exists():
                samples.unlink()
    base = out["no_rows"]["mean_iteration_ms"]
    for name in ("thin5", "thin1"):
        out[name]["overhead_ms_per_iteration"] = out[name]["mean_iteration_ms"] - base
    return out


def numpy_sample(m_sample, seed):
    """A CPU-generated sample of the workload: N individuals, m_sample markers."""
    from bayesrrcmd_gb300 import plink
    rng = np.random.default_rng(seed)
    p = rng.uniform(P_LO, P_HI, m_sample).astype(np.float32)
    g = np.zeros((m_sample, N_IND), np.int8)
    for j0 in range(0, m_sample, 256):
        j1 = min(m_sample, j0 + 256)
        pp = p[j0:j1, None]
        g[j0:j1] = (rng.random((j1 - j0, N_IND), dtype=np.float32) < pp).astype(np.int8) + \
                   (rng.random((j1 - j0, N_IND), dtype=np.float32) < pp).astype(np.int8)
    g[:, 0], g[:, 1] = 1, 0
    bed = plink.encode_bed(g)
    n_c = max(1, m_sample * N_CAUSAL // M_SNP)
    causal = rng.choice(m_sample, n_c, replace=False)
    b = rng.normal(0.0, np.sqrt(H2 / N_CAUSAL), n_c)
    x = plink.standardize_dense(g[causal])
    y = (b @ x + rng.normal(0.0, np.sqrt(1.0 - H2 * n_c / N_CAUSAL), N_IND)).astype(np.float32)
    group = (np.arange(m_sample) >= m_sample // 2).astype(np.int32)
    return bed, y, group


def cpu_reference(steps_ref, bed, y, group, warmup_ref=0):
    """FP64 restatement of the reference sampler on the host, on a sample of
    the markers of the workload (a sweep costs O(N) per marker, so the
    per-marker cost of the sample is that of the full M), one core: the
    reference's sampling node is serial.  The restatement is the build with
    the reference's fast release flags (-O3 -ffast-math -funroll-loops).
    warmup_ref untimed iterations come first."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_lib as O
    O.use_timing_build()
    m_sample = bed.shape[0]
    oc = O.OracleChain(np.ascontiguousarray(bed), N_IND, y, S_GROUPS, kind=0, group=group, seed=SEED)
    for it in range(warmup_ref):
        oc.iterate(it)
    t0 = time.perf_counter()
    for it in range(warmup_ref, warmup_ref + steps_ref):
        oc.iterate(it)
    dt = time.perf_counter() - t0
    return m_sample * steps_ref / dt, m_sample, dt


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-chain batching-form measurement")
    ap.add_argument("--batch-only", action="store_true",
                    help="only the batching-form leg (profiling); --batch-markers sets its M")
    ap.add_argument("--batch-markers", type=int, default=None)
    ap.add_argument("--no-uneven", action="store_true", help="skip the uneven-batch (32 regressions) measurement")
    ap.add_argument("--uneven-only", action="store_true", help="only the uneven-batch leg; --uneven-scale shrinks it")
    ap.add_argument("--uneven-scale", type=float, default=1.0)
    ap.add_argument("--no-ragged", action="store_true", help="skip the ragged (C2) and C1 measurements")
    ap.add_argument("--ragged-only", action="store_true",
                    help="only the ragged (C2) and C1 measurements (--no-cpu skips their CPU rates)")
    ap.add_argument("--sample-writer", action="store_true",
                    help="only the sample-file measurement: brr at the benchmark workload with and without rows")
    ap.add_argument("--matched-chains", action="store_true",
                    help="only the whole-chain comparisons of the chosen forms with the plain FP64 chain (C3: "
                         "1,000 iterations, burn-in 200; C2: 2,000 iterations, burn-in 500, thin 5)")
    ap.add_argument("--cluster-compare", action="store_true",
                    help="only the comparison of the grid-wide restart sweep with its thread-block-cluster variant "
                         "(C1, C2; C3 for two iterations)")
    ap.add_argument("--small", action="store_true",
                    help="profiling case: N=100,000 x M=8,192 (200 MB of codes, above L2), same settings")
    args = ap.parse_args()
    if args.small:
        global M_SNP, N_CAUSAL, WORKLOAD
        M_SNP, N_CAUSAL = 8192, 82
        WORKLOAD = WORKLOAD.replace("M=100,000", "M=8,192").replace("1,000 causal", "82 causal")

    rank, world, dist = dist_setup(args.gpus)
    if args.impl == "reference":
        if rank != 0:
            return
        # each step: one Gibbs iteration over a 5,000-marker sample (about 0.4 s on one core)
        m_sample = int(os.environ.get("BRR_REF_MARKERS", "5000"))
        bed, y, group = numpy_sample(m_sample, SEED)
        steps = args.steps
        rate, m_sample, dt = cpu_reference(steps, bed, y, group, warmup_ref=args.warmup)
        line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": "marker-updates/s",
                "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded numpy sample of the workload)",
                "config": {"workload": WORKLOAD, "sample_markers": m_sample},
                "cpu_baseline": {"value": rate, "unit": "marker-updates/s", "cores": 1, "kind": "port",
                                 "sample": f"{m_sample} markers x N={N_IND}, {steps} Gibbs iterations of the FP64 "
                                           f"restatement of the reference sampler built with the reference's fast "
                                           f"flags -O3 -ffast-math -funroll-loops ({dt:.1f} s); the reference "
                                           f"itself needs Eigen/Boost.Random/TBB, absent here"},
                "e2e": {"value": rate, "unit": "marker-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    from bayesrrcmd_gb300 import gpu
    from bayesrrcmd_gb300.build import build_gpu
    build_gpu()
    lib = gpu.load_library()
    device = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(device)
    if args.sample_writer:
        sw = run_sample_writer(lib, gpu, torch, device, int(os.environ.get("BRR_SW_ITERS", "60")))
        if rank == 0:
            print(json.dumps({"sample_writer": sw}))
        return
    if args.ragged_only:
        rr = run_ragged(lib, gpu, torch, device, args.steps, args.warmup, cpu=not args.no_cpu)
        if rank == 0:
            print(json.dumps({"ragged_only": True, **rr}))
        return
    if args.cluster_compare:
        cc = run_cluster_compare(lib, gpu, torch, device, args.steps, args.warmup)
        if rank == 0:
            print(json.dumps({"cluster_compare": cc}))
        return
    if args.matched_chains:
        mc = run_matched_chains(lib, gpu, torch, device, int(os.environ.get("BRR_C3_ITERS", "1000")),
                                int(os.environ.get("BRR_C2_ITERS", "2000")))
        if rank == 0:
            print(json.dumps({"matched_chains": mc}))
        return
    if args.uneven_only:
        uu = run_uneven(lib, gpu, torch, device, args.steps, 2, args.uneven_scale)
        if rank == 0:
            print(json.dumps({"uneven_only": True, **uu}))
        return
    if args.batch_only:
        global B_M
        if args.batch_markers:
            B_M = args.batch_markers
        bb = run_batched(lib, gpu, torch, device, args.steps, args.warmup)
        if rank == 0:
            print(json.dumps({"batched_only": True, "markers": B_M, "value": bb["rate"], "unit": "marker-updates/s",
                              "aggregate_vs_plain": bb["rate"] / bb["plain"], "ms_per_step": bb["ms_per_step"],
                              "alg_tflops": bb["alg_tflops"], "cycles_per_block": bb["cycles"]}))
        return
    d_bed, y, group = make_problem(lib, gpu, torch, device, rank)

    def barrier():
        torch.cuda.synchronize(device)
        if dist:
            dist.barrier()

    barrier()
    with ClockSampler(device) as clk:
        fp32c = run_form(lib, gpu, torch, device, d_bed, y, group, gpu.FORM_FP32C, args.steps, args.warmup, rank,
                         barrier, profile=True)
    barrier()
    fp64 = run_form(lib, gpu, torch, device, d_bed, y, group, gpu.FORM_FP64, args.steps, args.warmup, rank,
                    barrier)
    barrier()
    t_chosen = max_over_ranks(fp32c["total_ms"] / 1e3, dist, device)
    value = replica_rate(world, M_SNP, args.steps, t_chosen)
    host_t = torch.empty(d_bed.numel(), dtype=torch.uint8, pin_memory=True)
    host_t.copy_(d_bed)
    host_bed = host_t.numpy()
    e2e = None
    if not args.no_e2e:
        # a chain as a user runs one (the workload's configuration runs 1,000 iterations): the
        # one-time upload, packing and marker-Gram build are paid once per chain
        e2e_steps = int(os.environ.get("BRR_E2E_STEPS", "200"))
        e = run_e2e(lib, gpu, torch, device, host_bed, y, group, e2e_steps, rank)
        e2e = {"value": replica_rate(world, M_SNP, e2e_steps, max_over_ranks(e["wall"], dist, device)),
               "unit": "marker-updates/s",
               "h2d_bytes_per_step": int(e["h2d_per_step"]), "d2h_bytes_per_step": int(e["d2h_per_step"]),
               "includes": f"chain of {e2e_steps} iterations: pinned-host BED upload + device packing + "
                           f"marker Gram + init, then per iteration the sample read-back",
               "parts_s": e["parts"]}
    batched = None
    if not args.no_batch and not args.small:
        bsteps = int(os.environ.get("BRR_BATCH_STEPS", "3"))
        bb = run_batched(lib, gpu, torch, device, bsteps, max(args.warmup, 2))
        bf16_peak = peaks_bf16()
        batched = {
            "workload": B_WORKLOAD,
            "value": replica_rate(world, B_C * B_M, bsteps, max_over_ranks(bb["total_s"], dist, device)),
            "unit": "marker-updates/s (all chains)",
            "chains": B_C, "steps": bsteps, "ms_per_step": bb["ms_per_step"], "sweep_ms": bb["sweep_ms"],
            "plain_fp64_same_genotypes": {"value": bb["plain"], "unit": "marker-updates/s (one chain)",
                                          "ms_per_step": bb["plain_ms"]},
            "aggregate_vs_plain": bb["rate"] / bb["plain"],
            "roofline": {"bound": "tensor", "achieved": bb["alg_tflops"], "peak": bf16_peak, "unit": "TFLOP/s",
                         "frac": bb["alg_tflops"] / bf16_peak, "traffic": None,
                         "issued_tflops": bb["issued_tflops"], "kernel": "k_sweep_batch (tcgen05 kind::f16)",
                         "note": "algorithmic FLOPs: X_block^T E, X_block dB and the block Gram"},
            "phase_clk_per_block_cta0": dict(zip(["dots", "publish", "resolve", "update", "resolve_wait_dots",
                                                  "resolve_chain0", "steps_chain0", "resolve_wait_slowest"],
                                                 bb["cycles"])),
            "geometry": bb["geometry"],
        }
    uneven = None
    if not args.no_uneven and not args.small:
        usteps = int(os.environ.get("BRR_UNEVEN_STEPS", "3"))
        uu = run_uneven(lib, gpu, torch, device, usteps, 2)
        u_value = replica_rate(world, uu["total_markers"], usteps, max_over_ranks(uu["total_s"], dist, device))
        uneven = {"workload": U_WORKLOAD, "value": u_value,
                  "unit": "marker-updates/s (all instances)", "steps": usteps, "ms_per_step": uu["ms_per_step"],
                  "sweep_ms": uu["sweep_ms"], "instances": uu["instances"], "total_markers": uu["total_markers"],
                  "total_genotypes": uu["total_genotypes"], "kinds": uu["kinds"],
                  "autotuner": {"ctas_initial": uu["ctas_first"], "ctas": uu["ctas"], "round_widths": uu["widths"],
                                "instance_sweep_ms": uu["inst_ms"],
                                "slowest_over_mean": uu["balance_max_over_mean"]},
                  "sizes": {"N": uu["N"], "M": uu["M"]}}
    ragged = None
    if not args.no_ragged and not args.small:
        ragged = run_ragged(lib, gpu, torch, device, int(os.environ.get("BRR_RAGGED_STEPS", "10")), 3,
                            cpu=not args.no_cpu and rank == 0)
        ragged["value"] = replica_rate(world, R_M, ragged["steps"],
                                       max_over_ranks(ragged["ms_per_step"] * ragged["steps"] / 1e3, dist, device))
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu:
        m_sample = min(M_SNP, int(os.environ.get("BRR_REF_MARKERS", "20000")))
        it_sample = 8
        bed_s = host_bed.reshape(M_SNP, -1)[:m_sample]
        rate, m_sample, dt = cpu_reference(it_sample, bed_s, y, group[:m_sample])
        cpu = {"value": rate, "unit": "marker-updates/s", "cores": 1, "kind": "port",
               "sample": f"first {m_sample} markers x N={N_IND} of the same data, {it_sample} Gibbs iterations of "
                         f"the FP64 restatement of the reference sampler built with the reference's fast flags "
                         f"-O3 -ffast-math -funroll-loops ({dt:.1f} s)"}
    hbm, peak_kind = peaks()
    sweep_s = fp32c["sweep_ms"] / 1e3 / args.steps
    bytes_per_sweep = M_SNP * (N_IND / 4.0)      # 2-bit genotype bytes per marker-update x M
    achieved = bytes_per_sweep / sweep_s / 1e9
    # DRAM bytes of one blocked-sweep launch, measured by ncu on the N=100,000 x
    # M=8,192 case (dram__bytes.sum.per_second x gpu__time_duration.sum = 295.0 MB),
    # scaled by the markers swept (the traffic grows with M at fixed N)
    traffic = DRAM_BYTES_PER_MARKER_N100K * M_SNP if N_IND == 100_000 else None
    plain_rate = M_SNP * args.steps / (fp64["total_ms"] / 1e3)
    nzb = fp64["beta"] != 0
    line = {
        "metric": METRIC, "value": value, "unit": "marker-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": fp32c["total_ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 compensated (FP64 refresh, FP64 log-likelihoods)",
        "data": "synthetic (seeded, generated on the device)",
        "config": {"workload": WORKLOAD, "form": "fp32c" + (" gram-blocked" if fp32c["gram"]["blocked"] else ""),
                   "refresh_every": REFRESH,
                   "l2": f"inputs larger than L2 ({M_SNP * N_IND / 4 / 1e9:.2g} GB of codes per sweep)", "parallelism": "replicas" if world > 1 else "1 chain"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback 6.8 TB/s",
                     "kernel": "k_sweep_block (FP32C dense, Gram-blocked)",
                     "algorithmic_bytes_per_launch": bytes_per_sweep},
        "phases_clk_per_round": {k: v / max(fp32c["phases"][5], 1) for k, v in
                                 zip(["ring_wait", "dot_side", "barrier_wait", "sample", "update", "block_inputs",
                                      "of_sample_picks", "of_sample_steps", "next_block_inputs"],
                                     [*fp32c["phases"][:5], fp32c["phases"][7], *fp32c["phases"][9:12]])},
        "phases_source": f"{PROFILE_STEPS} iterations of the phase-counting kernel variant after the timed steps",
        "role_end_clk_per_round": {k: fp32c["phases"][i] / max(fp32c["phases"][5], 1)
                                   for k, i in (("dot_warps", 12), ("gram_warp", 13), ("resolve_warp", 14),
                                                ("input_warp", 15))},
        "sampling_steps_per_round": fp32c["phases"][6] / max(fp32c["phases"][5], 1),
        "fp64_fallbacks_per_step": fp32c["phases"][8] / PROFILE_STEPS,
        "rounds_per_step": fp32c["rounds"] / args.steps,
        "gram": {"blocked_sweep": fp32c["gram"]["blocked"], "build_ms": fp32c["gram"]["build_ms"],
                 "gemm_operand_bits": fp32c["gram"].get("operand_bits"),
                 "bytes": fp32c["gram"]["bytes"]},
        "gpu_launches": 5 * args.steps + (args.steps + args.warmup) // REFRESH,
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
        "e2e": e2e,
        "batched": batched,
        "uneven": uneven,
        "ragged": ragged,
        "plain_fp64": {"value": plain_rate, "unit": "marker-updates/s", "ms_per_step": fp64["total_ms"] / args.steps,
                       "speedup_chosen_vs_plain": value / world / plain_rate,
                       "rounds_per_step": fp64["rounds"] / args.steps},
        "matched_error": {"beta_max_abs_diff_vs_plain": float(np.abs(fp32c["beta"] - fp64["beta"]).max()),
                          "sigmaE_rel_diff_vs_plain": abs(fp32c["sigmaE"] / fp64["sigmaE"] - 1),
                          "sigmaG_max_rel_diff_vs_plain": float(np.max(np.abs(np.asarray(fp32c["sigmaG"]) /
                                                                               np.asarray(fp64["sigmaG"]) - 1))),
                          "component_mismatches_vs_plain": int(np.count_nonzero(fp32c["comp"] != fp64["comp"])),
                          "component_counts_plain": np.bincount(fp64["comp"], minlength=4).tolist(),
                          "compared": "final state after the warm-up and timed iterations (same draws)",
                          "nonzero_beta_plain": int(nzb.sum())},
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
