"""Benchmark: batched Metropolis integration of a correlated 16-D Gaussian (C2).

Workload (one "step" = one full MCI::integrate over every chain):
  65,536 independent chains, ndim 16, target N(0, Sigma) with
  Sigma = Q diag(lambda) Q^T, Q a seeded random orthogonal matrix (QR of a
  standard normal matrix, sign-fixed) and lambda log-uniform on [0.1, 10];
  Gaussian all-coordinate move with per-chain step calibration to 50 %
  acceptance (automatic findMRT2Step), 1,000 burn-in steps, 10,000 sampling
  steps; observables x.x (analytic mean tr Sigma) and x_i, each stored twice:
  FullAccumulator with float samples and BlockAccumulator with 100 blocks.
  float walker arithmetic, Kahan-compensated float block sums.

Metric: effective samples/s of <x.x>, ESS = Var(x.x) / err^2 where
Var(x.x) = 2 tr(Sigma^2) is the target variance and err the integrator's
combined standard error from the 100-block accumulator (the reference's
Uncorrelated estimator on block means, combined over chains with the MPIMCI
formula).  `value` times the device work with inputs resident; `e2e` times the
same integrate through the C ABI with the initial walkers copied from pinned
host memory and the averages / errors read back every step.

--impl reference times the CPU path on the host cores: the oracle's
restatement of the reference (one reference MCI per chain, std::mt19937_64
draws, double arithmetic) on a bounded sample of chains, all host threads.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NDIM = 16
NCHAINS = 65536
NMC = 10000
BURNIN = 1000
NBLOCKS = 100
METRIC = "effective samples/s of <x.x> (C2: 65,536 chains x 16-D correlated Gaussian, plain MH)"


def target(seed=2024):
    rng = np.random.default_rng(seed)
    Q, R = np.linalg.qr(rng.standard_normal((NDIM, NDIM)))
    Q = Q * np.sign(np.diag(R))
    lam = 10.0 ** rng.uniform(-1.0, 1.0, NDIM)
    Sigma = Q @ np.diag(lam) @ Q.T
    P = Q @ np.diag(1.0 / lam) @ Q.T
    return Sigma, 0.5 * (P + P.T)


def configure(m, P, nmc):
    """Same configuration for the device MCI and the oracle (MCI-style API)."""
    m.add_sampling_function(3, P)            # GAUSS_PREC
    m.set_trial_move(0, 1, 0)                # all-coordinate, Gaussian
    m.set_nfind_mrt2_iterations(-50)
    m.set_ndecorrelation_steps(BURNIN)
    bs = nmc // NBLOCKS
    m.add_observable(0, (), bs, 1, False, 1)  # x.x, Block, Uncorrelated
    m.add_observable(1, (), bs, 1, False, 1)  # x_i, Block, Uncorrelated
    m.add_observable(0, (), 1, 1, False, 1)   # x.x, Full
    m.add_observable(1, (), 1, 1, False, 1)   # x_i, Full


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self):
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200", "-i", "0"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([v.strip() for v in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": len(self.samples)}
        sm = [float(s[0]) for s in self.samples if len(s) >= 8 and s[0].replace(".", "").isdigit()]
        if sm:
            out["sm_mhz"] = float(np.median(sm))
            out["sm_max_mhz"] = float(self.samples[0][1])
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            seen = set()
            for s in self.samples:
                for k, n in enumerate(names):
                    if len(s) > 4 + k and s[4 + k].lower().startswith("active"):
                        seen.add(n)
            out["reasons"] = sorted(seen)
        return out


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def run_gpu(args):
    import torch
    import mcintegratorplusplus_gb300 as mcig

    Sigma, P = target()
    var_xx = 2.0 * float(np.trace(Sigma @ Sigma))
    nchains = args.chains
    m = mcig.MCI(NDIM, nchains, device=0, precision=mcig.PREC_FP32)
    m.setSeed(20241203)
    m.setFullStorage(32)
    configure(m, P, args.nmc)
    nod = m.getNObsDim()
    # pinned host buffers: initial walkers in, averages / errors out
    x0 = torch.zeros((nchains, NDIM), dtype=torch.float64).pin_memory()
    avg = torch.zeros(nod, dtype=torch.float64).pin_memory()
    err = torch.zeros(nod, dtype=torch.float64).pin_memory()
    avg_np, err_np = avg.numpy(), err.numpy()
    l2flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def one_step(timed_e2e):
        if timed_e2e:
            m.setX(x0.numpy())  # host -> device copy of the step's input walkers
        m.integrate_into(args.nmc, avg_np, err_np)
        return m.getLastTimings()

    for _ in range(args.warmup):
        one_step(True)
        l2flush.zero_()
    torch.cuda.synchronize()

    clocks = Clocks()
    clocks.start()
    dev_ms, wall = [], []
    kernel_ms = []
    launches = 0
    for _ in range(args.steps):
        l2flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tm = one_step(True)
        t1 = time.perf_counter()
        wall.append(t1 - t0)
        dev_ms.append(tm["calibration_ms"] + tm["burnin_ms"] + tm["sampling_ms"] + tm["estimation_ms"])
        kernel_ms.append(tm["sampling_ms"])
        launches += tm["launches"]
    torch.cuda.synchronize()
    ck = clocks.stop()

    xx, exx = float(avg_np[0]), float(err_np[0])
    ess = var_xx / (exx * exx)
    ms_dev = float(np.mean(dev_ms))
    ms_e2e = float(np.mean(wall)) * 1e3
    steps_total = nchains * (args.nmc)
    # dominant kernel: the sampling launch (float Full stores + block sums)
    samp_ms = float(np.mean(kernel_ms))
    full_bytes = nchains * args.nmc * (1 + NDIM) * 4       # Full float stores
    block_bytes = nchains * NBLOCKS * (1 + NDIM) * 8       # Block means (double)
    state_bytes = nchains * (NDIM * 8 * 2 + 8 * 4)         # walker in/out, step, counter
    algo_bytes = full_bytes + block_bytes + state_bytes
    pk, pk_kind = peaks()
    achieved = algo_bytes / (samp_ms * 1e-3) / 1e9
    flop_per_step = 2 * (NDIM * (NDIM + 1) // 2 + NDIM) + 2 * NDIM + 4 * (1 + NDIM) + 2 * NDIM
    line = {
        "metric": METRIC, "value": ess / (ms_dev * 1e-3), "unit": "effective samples/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_dev,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded correlated Gaussian target, random-init walkers at 0)",
        "config": {"workload": "C2 batched plain Metropolis", "chains": nchains, "ndim": NDIM,
                   "nmc": args.nmc, "burnin": BURNIN, "blocks": NBLOCKS, "full_storage": "f32",
                   "accumulation": "f32+Kahan", "calibration": "auto per chain (target 0.5)",
                   "l2": "flushed (256 MB write) before each step; Full output > L2"},
        "walker_steps_per_s": steps_total / (ms_dev * 1e-3),
        "estimate": {"x.x": xx, "err": exx, "tr_sigma": float(np.trace(Sigma)),
                     "z": (xx - float(np.trace(Sigma))) / exx, "acceptance": m.getAcceptanceRate()},
        "phases_ms": {k: float(v) for k, v in tm.items() if k.endswith("_ms")},
        "e2e": {"value": ess / (ms_e2e * 1e-3), "unit": "effective samples/s",
                "h2d_bytes_per_step": int(x0.numel() * 8), "d2h_bytes_per_step": int(2 * nod * 8),
                "ms_per_step": ms_e2e},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": float(pk["hbm_gbs"]), "unit": "GB/s",
                     "frac": achieved / float(pk["hbm_gbs"]), "traffic": None, "peak_source": pk_kind,
                     "kernel": "sampling launch (mcig_fast_kernel<16,ALL,Kahan>)",
                     "algorithmic_bytes_per_launch": algo_bytes, "kernel_ms": samp_ms,
                     "fp32_flop_per_step": flop_per_step},
        "gpu_launches": launches,
        "clocks": ck,
    }
    if args.cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args)
    return line


def cpu_baseline(args):
    """The oracle (reference restated: std::mt19937_64, double, one MCI per chain) on host threads."""
    from oracle import oracle as orc
    Sigma, P = target()
    var_xx = 2.0 * float(np.trace(Sigma @ Sigma))
    nthreads = os.cpu_count() or 1
    nch = max(nthreads, args.cpu_chains)
    m = orc.OracleMCI(NDIM, nch)
    m.set_seeds(np.arange(1, nch + 1, dtype=np.uint64) * 7919)
    configure(m, P, args.nmc)
    t0 = time.perf_counter()
    avg, err = m.integrate(args.nmc, True, True, nthreads=nthreads)
    dt = time.perf_counter() - t0
    # the full workload has NCHAINS chains: error scales as 1/sqrt(chains), time as chains/threads
    ess_sample = var_xx / float(err[0]) ** 2
    return {"value": ess_sample / dt, "unit": "effective samples/s", "cores": nthreads, "kind": "port",
            "sample": "%d of the %d chains, full length (calibration, %d burn-in, %d steps), %.1f s" %
                      (nch, NCHAINS, BURNIN, args.nmc, dt),
            "walker_steps_per_s": nch * args.nmc / dt, "x.x": float(avg[0]), "err": float(err[0])}


def run_reference(args):
    cb = None
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(args)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cb = cpu_baseline(args)
        vals.append(cb["value"])
    dt = (time.perf_counter() - t0) / max(args.steps, 1)
    v = float(np.mean(vals))
    return {"metric": METRIC, "value": v, "unit": "effective samples/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "C2 batched plain Metropolis", "chains_sampled": cb and cb["sample"],
                       "ndim": NDIM, "nmc": args.nmc},
            "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "effective samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--chains", type=int, default=NCHAINS)
    ap.add_argument("--nmc", type=int, default=NMC)
    ap.add_argument("--cpu-chains", type=int, default=32)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return
    if world > 1:  # replicas only: every rank runs its own chains, rank 0 reports the max-time aggregate
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
        line = run_gpu(args)
        t = torch.tensor([line["ms_per_step"], line["e2e"]["ms_per_step"]], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        if rank == 0:
            ess_rank = line["value"] * line["ms_per_step"] * 1e-3
            line["value"] = ess_rank * world / (float(t[0]) * 1e-3)
            line["e2e"]["value"] = ess_rank * world / (float(t[1]) * 1e-3)
            line["n_gpus"] = world
            line["ms_per_step"] = float(t[0])
            print(json.dumps(line), flush=True)
        dist.destroy_process_group()
        return
    print(json.dumps(run_gpu(args)), flush=True)


if __name__ == "__main__":
    main()
