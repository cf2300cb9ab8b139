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
Var(x.x) = 2 tr(Sigma^2) is the target variance and err the standard error of the
combined estimate measured from the spread of the chain means (the chains are
independent: err^2 = var(chain means) / nchains), so ESS = nchains * NMC / (2 tau_int).
Two estimates of the integrated autocorrelation time tau_int of x.x check it, from the
Full samples of 256 chains: the reference's MJBlocker (src/MJBlocker.cpp:127-154) on
the last 8,192 samples of every chain, and Sokal's self-consistent window (c = 5) on
the chain-averaged autocorrelation.  The 100-block error that the integrator reports
(Uncorrelated estimator on block means) is kept as a labelled diagnostic: with tau_int
above the 100-step block length it underestimates the error.  `value` times the device
work with inputs resident; `e2e` times the same integrate through the C ABI with the
initial walkers copied from pinned host memory and the averages / errors read back
every step.

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
METRIC = "effective samples/s on 1 GB300 at matched std-error: learned/batched vs plain MH"
# ncu figures of the sampling launch (65,536 chains, 600 steps, 6 blocks of 100, four
# accumulators): DRAM bytes read + written, and warp instructions per warp-step
CAPTURE_DRAM_BYTES = 9.70e6 + 2.6774e9
INST_PER_WARP_STEP = 851.0


def target(seed=2024):
    rng = np.random.default_rng(seed)
    Q, R = np.linalg.qr(rng.standard_normal((NDIM, NDIM)))
    Q = Q * np.sign(np.diag(R))
    lam = 10.0 ** rng.uniform(-1.0, 1.0, NDIM)
    Sigma = Q @ np.diag(lam) @ Q.T
    P = Q @ np.diag(1.0 / lam) @ Q.T
    return Sigma, 0.5 * (P + P.T)


def configure(m, P, nmc, nblocks=NBLOCKS):
    """Same configuration for the device MCI and the oracle (MCI-style API)."""
    m.add_sampling_function(3, P)            # GAUSS_PREC
    m.set_trial_move(0, 1, 0)                # all-coordinate, Gaussian
    m.set_nfind_mrt2_iterations(-50)
    m.set_ndecorrelation_steps(BURNIN)
    bs = nmc // nblocks
    m.add_observable(0, (), bs, 1, False, 1)  # x.x, Block, Uncorrelated
    m.add_observable(1, (), bs, 1, False, 1)  # x_i, Block, Uncorrelated
    m.add_observable(0, (), 1, 1, False, 1)   # x.x, Full
    m.add_observable(1, (), 1, 1, False, 1)   # x_i, Full


def sokal_tau(series, c=5.0):
    """Integrated autocorrelation time of series[nchains][n] (steps): chain-averaged
    autocorrelation, tau(M) = 1/2 + sum_{t=1..M} rho(t), smallest M >= c tau(M)."""
    x = np.asarray(series, dtype=np.float64)
    x = x - x.mean(axis=1, keepdims=True)
    n = x.shape[1]
    f = np.fft.rfft(x, 2 * n, axis=1)
    acf = np.fft.irfft(f * np.conj(f), axis=1)[:, :n].mean(axis=0) / np.arange(n, 0, -1)
    rho = acf / acf[0]
    tau = 0.5 + np.cumsum(rho[1:])
    for M in range(1, n - 1):
        if M >= c * tau[M - 1]:
            return float(tau[M - 1])
    return float(tau[-1])


def ess_report(chain_means, var, nchains, nmc, series=None, mj=None, block_err=None):
    """Effective sample size of the combined mean from the spread of the chain means, with
    tau_int cross-checks on a few chains' full series (mj: MJBlocker estimator function
    taking x[n][ndim] and returning (avg[ndim], err[ndim]))."""
    cm = np.asarray(chain_means, dtype=np.float64)
    err_bc = float(cm.std(ddof=1) / np.sqrt(len(cm)))
    ess = var / err_bc ** 2 * (nchains / len(cm))
    out = {"ess": ess, "err_between_chains": err_bc, "tau_int_between_chains": nchains * nmc / (2.0 * ess),
           "definition": "ESS = Var / err^2, Var the target variance of the observable, err = std(chain means) / sqrt(chains)"}
    if series is not None:
        s = np.asarray(series, dtype=np.float64)
        out["tau_int_sokal"] = sokal_tau(s)
        out["tau_series"] = "Full samples of the observable, %d chains x %d" % s.shape
        if mj is not None:
            n2 = 1 << int(np.floor(np.log2(s.shape[1])))
            tail = np.ascontiguousarray(s[:, -n2:].T)  # [n2][chains]: one MJBlocker series per chain
            _, e = mj(tail)
            v = tail.var(axis=0, ddof=1)
            out["tau_int_mjblocker"] = float(np.mean(n2 * np.asarray(e) ** 2 / (2.0 * v)))
            out["mjblocker_samples"] = n2
        taus = [out[k] for k in ("tau_int_sokal", "tau_int_mjblocker") if k in out]
        out["ess_over_ess_from_tau"] = [float(nchains * nmc / (2.0 * t) / ess) for t in taus]
    if block_err is not None:
        out["block100_err_over_between_chain_err"] = float(block_err / err_bc)
        out["ess_block100_diagnostic"] = float(var / block_err ** 2)
    return out


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
                 "--format=csv,noheader,nounits", "-lms", "50", "-i", "0"],
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
    configure(m, P, args.nmc, args.blocks)
    if args.c2_kernel == "one-lane":
        m.setKernel(2)
    elif args.c2_kernel == "pair":
        m.setLanes(2)
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
        launches += tm["launches"] + 1  # integrate's launches and setX's transpose of the walkers
    torch.cuda.synchronize()
    ck = clocks.stop()

    xx, exx = float(avg_np[0]), float(err_np[0])
    ca, _ = m.getChainResults()
    ntau = min(256, nchains)
    rep = ess_report(ca[:, 0], var_xx, nchains, args.nmc, series=m.getObsDataChains(2, 0, ntau),
                     mj=lambda x: mcig.estimate(mcig.EST_MJBLOCKER, x), block_err=exx)
    ess = rep["ess"]
    ms_dev = float(np.mean(dev_ms))
    ms_e2e = float(np.mean(wall)) * 1e3
    steps_total = nchains * (args.nmc)
    # dominant kernel: the sampling launch (float Full stores + block sums)
    samp_ms = float(np.mean(kernel_ms))
    full_bytes = nchains * args.nmc * (1 + NDIM) * 4       # Full float stores
    block_bytes = nchains * args.blocks * (1 + NDIM) * 8   # Block means (double)
    state_bytes = nchains * (NDIM * 8 * 2 + 8 * 4)         # walker in/out, step, counter
    algo_bytes = full_bytes + block_bytes + state_bytes
    pk, pk_kind = peaks()
    achieved = algo_bytes / (samp_ms * 1e-3) / 1e9
    traffic = CAPTURE_DRAM_BYTES * (nchains / 65536.0) * (args.nmc / 600.0)
    # instruction-issue bound: 4 warp-instructions per cycle per SM, 152 SMs
    sm_mhz = ck["sm_mhz"] or float(pk.get("sm_max_mhz", 2070.0))
    warp_steps = nchains / 32.0 * args.nmc
    issue_ms = INST_PER_WARP_STEP * warp_steps / (152 * 4 * sm_mhz * 1e6) * 1e3
    flop_per_step = 2 * (NDIM * (NDIM + 1) // 2 + NDIM) + 2 * NDIM + 4 * (1 + NDIM) + 2 * NDIM
    line = {
        "metric": METRIC, "value": ess / (ms_dev * 1e-3), "unit": "effective samples/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_dev,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded correlated Gaussian target, random-init walkers at 0)",
        "config": {"workload": "C2 batched plain Metropolis", "chains": nchains, "ndim": NDIM,
                   "nmc": args.nmc, "burnin": BURNIN, "blocks": args.blocks, "full_storage": "f32",
                   "accumulation": "f32+Kahan", "calibration": "auto per chain (target 0.5)",
                   "l2": "flushed (256 MB write) before each step; Full output > L2"},
        "walker_steps_per_s": steps_total / (ms_dev * 1e-3),
        "estimate": {"x.x": xx, "err_block100": exx, "err_between_chains": rep["err_between_chains"],
                     "tr_sigma": float(np.trace(Sigma)),
                     "z": (xx - float(np.trace(Sigma))) / rep["err_between_chains"],
                     "acceptance": m.getAcceptanceRate()},
        "ess": rep,
        "phases_ms": {k: float(v) for k, v in tm.items() if k.endswith("_ms")},
        "e2e": {"value": ess / (ms_e2e * 1e-3), "unit": "effective samples/s",
                "h2d_bytes_per_step": int(x0.numel() * 8), "d2h_bytes_per_step": int(2 * nod * 8),
                "ms_per_step": ms_e2e},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": float(pk["hbm_gbs"]), "unit": "GB/s",
                     "frac": achieved / float(pk["hbm_gbs"]), "traffic": traffic, "peak_source": pk_kind,
                     "traffic_source": "ncu dram__bytes_read+write of a 600-step capture of this launch "
                                       "(65,536 chains), scaled by chains x steps",
                     "kernel": "sampling launch (mcig_fast_kernel<16,ALL,Kahan,PREC,moments,lean Gaussian,fixed4>)",
                     "algorithmic_bytes_per_launch": algo_bytes, "kernel_ms": samp_ms,
                     "fp32_flop_per_step": flop_per_step},
        "issue_roofline": {"bound": "instruction issue", "warp_inst_per_warp_step": INST_PER_WARP_STEP,
                           "issue_limited_ms": issue_ms, "kernel_ms": samp_ms, "frac": issue_ms / samp_ms,
                           "sm_mhz": sm_mhz, "source": "ncu smsp__inst_executed.sum of the same capture"},
        "gpu_launches": launches,
        "clocks": ck,
    }
    if args.batched:
        c3 = run_c3(argparse.Namespace(integrals=4096, warmup=1, steps=3, c3_tuning=getattr(args, "c3_tuning", None)))
        line["batched"] = {"workload": c3["metric"], "integrals_per_s": c3["value"], "ms_per_batch": c3["ms_per_step"],
                           "e2e_integrals_per_s": c3["e2e"]["value"], "outer_steps_per_s": c3["outer_steps_per_s"],
                           "config": c3["config"], "accuracy": c3["accuracy"], "clocks": c3["clocks"]}
    if args.learned:
        c5 = run_c5(argparse.Namespace(chains5=16384, nmc5=8192, warmup=1, steps=1, c5_flow_gemm=args.c5_flow_gemm))
        line["learned_proposal"] = {
            "workload": "C5: 16,384 chains x 24-D 4-mode mixture, 8-layer affine-coupling flow every 5th step",
            "ess_per_s_flow": c5["value"], "ess_per_s_plain_mh": c5["plain_mh"]["value"],
            "ratio": c5["ess_per_s_ratio_flow_over_plain"], "flow_acceptance": c5["flow"]["acceptance"],
            "ms_flow": c5["ms_per_step"], "ms_plain": c5["plain_mh"]["ms_per_step"], "flow_gemms": c5["flow_gemms"]}
    if args.cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args)
    return line


def cpu_baseline(args, target_s=10.0):
    """The oracle (reference restated: std::mt19937_64, double, one MCI per chain) on host threads.

    A pilot of 2 chains per thread sets the chain count so that the sample takes about
    `target_s` seconds of wall time on all host threads."""
    from oracle import oracle as orc
    Sigma, P = target()
    var_xx = 2.0 * float(np.trace(Sigma @ Sigma))
    nthreads = os.cpu_count() or 1

    def sample(nch):
        m = orc.OracleMCI(NDIM, nch)
        m.set_seeds(np.arange(1, nch + 1, dtype=np.uint64) * 7919)
        configure(m, P, args.nmc, args.blocks)
        t0 = time.perf_counter()
        avg, err, ca, _ = m.integrate(args.nmc, True, True, nthreads=nthreads, per_chain=True)
        return m, avg, err, ca, time.perf_counter() - t0

    nch = max(2 * nthreads, args.cpu_chains)
    m, avg, err, ca, dt = sample(nch)
    if dt < 0.5 * target_s:
        nch = int(min(NCHAINS, max(nch, nch * target_s / max(dt, 1e-3)) // nthreads * nthreads))
        del m
        m, avg, err, ca, dt = sample(nch)
    # ESS is proportional to the number of chains, so ESS/s of the sample is that of the full workload
    ntau = min(256, nch)
    series = m.obs_data(2)[:ntau]
    rep = ess_report(ca[:, 0], var_xx, nch, args.nmc, series=series,
                     mj=lambda x: orc.estimate(4, x), block_err=float(err[0]))
    return {"value": rep["ess"] / dt, "unit": "effective samples/s", "cores": nthreads, "kind": "port",
            "sample": "%d of the %d chains, full length (calibration, %d burn-in, %d steps), %.1f s" %
                      (nch, NCHAINS, BURNIN, args.nmc, dt),
            "walker_steps_per_s": nch * args.nmc / dt, "x.x": float(avg[0]), "err_block100": float(err[0]),
            "chains": nch, "ess": rep}


def run_reference(args):
    cb = None
    vals = []
    for _ in range(args.warmup):
        args.cpu_chains = cpu_baseline(args)["chains"]  # the first call sizes the sample
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


# ---------------------------------------------------------------------------
# further workloads (--workload c3|c4|c5); the default line is the C2 workload
# ---------------------------------------------------------------------------

def _timed_device_ms(tm):
    return tm["calibration_ms"] + tm["burnin_ms"] + tm["sampling_ms"] + tm["estimation_ms"]


def c3_integrals(n, steps=16384, seed=33):
    """The uneven batch: integral i has ndim ~ U{1..64}, NMC_i = 2^U(14,20) samples, a product of
    2-4 isotropic Gaussians on contiguous coordinate blocks (widths log-uniform on [0.3, 3]) as
    sampling functions and as the MultiStepMove's sub-pdfs (4 single-coordinate sub-moves), and
    x.x per block in a BlockAccumulator (16 blocks per chain).  The NMC_i samples are split over
    ceil(NMC_i / steps) chains (MPIMCI-style), each with a 500-step burn-in, so that the GPU has
    tens of thousands of chains to run; one chain of the whole NMC_i per integral would leave
    most of the GPU idle (4,096 chains are 0.8 warps per SM)."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n):
        ndim = int(rng.integers(1, 65))
        nmc_total = int(round(2 ** rng.uniform(14, 20)))
        nch = max(1, -(-nmc_total // steps))
        nmc = 16 * (-(-nmc_total // (16 * nch)))
        nb = int(min(ndim, rng.integers(2, 5)))
        cuts = np.sort(rng.choice(np.arange(1, ndim), nb - 1, replace=False)) if nb > 1 else np.array([], int)
        bounds = [0] + [int(c) for c in cuts] + [ndim]
        widths = 10.0 ** rng.uniform(np.log10(0.3), np.log10(3.0), nb)
        specs.append((ndim, nch, nmc, bounds, widths))
    return specs


def run_c3(args):
    """4,096 uneven integrals in one batch: ONE persistent launch (block-separable sampler,
    walkers in shared memory) captured in a CUDA graph with the estimators and the read-back,
    tuned by the autotuner (threads per block, sub-step unroll per ndim bucket).  Step
    calibration is off: with the MultiStepMove's sub-chain on the full target every outer step
    is accepted, and the reference's findMRT2Step would double the sub-move step on every
    iteration; the sub-move step is 2 x the geometric mean width.  Metric: integrals/s."""
    import mcintegratorplusplus_gb300 as mcig
    specs = c3_integrals(args.integrals)
    mcis, exact, nmcs, chains = [], [], [], []
    for i, (ndim, nch, nmc, bounds, widths) in enumerate(specs):
        nb = len(widths)
        m = mcig.MCI(ndim, nch, precision=mcig.PREC_FP32)
        m.setSeed(1000 + i)
        for k in range(nb):
            m.addSamplingFunction(mcig.PDF_GAUSS_BLOCK, [bounds[k], bounds[k + 1], widths[k]])
        m.setMultiStepMove(4, mcig.SRRD_UNIFORM, 1, float(2.0 * np.exp(np.mean(np.log(widths)))))
        for k in range(nb):
            m.addMultiStepSamplingFunction(mcig.PDF_GAUSS_BLOCK, [bounds[k], bounds[k + 1], widths[k]])
        m.setNfindMRT2Iterations(0)
        m.setNdecorrelationSteps(500)
        m.addObservable(mcig.OBS_X2BLOCK, [nb] + bounds, nmc // 16, 1, False, mcig.EST_UNCORRELATED)
        mcis.append(m)
        exact.append(np.array([(bounds[k + 1] - bounds[k]) * widths[k] ** 2 for k in range(nb)]))
        nmcs.append(nmc)
        chains.append(nch)
    b = mcig.Batch(mcis, nmcs)
    if getattr(args, "c3_tuning", None):
        v = [int(t) for t in args.c3_tuning.split(",")]
        b.set_tuning(v[0], v[1:5])
        block, unroll = b.tuning()
    else:
        block, unroll = b.autotune(None)
    for _ in range(args.warmup):
        b.run()
    clocks = Clocks()
    clocks.start()
    ms, wall = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        b.run()
        wall.append(time.perf_counter() - t0)
        ms.append(b.last_ms())
    ck = clocks.stop()
    # accuracy against the analytic block moments: z from the chains' own block errors
    # (16 blocks of >= 1,024 steps, far above tau_int here) for every integral, and z from the
    # spread of the chain means for integrals with >= 8 chains (with 2-7 chains that spread
    # has too few degrees of freedom for a 3-sigma test)
    z, zs = [], []
    for m, x in zip(mcis, exact):
        ca, ce = m.getChainResults()
        nc = ca.shape[0]
        z.append(np.abs(ca.mean(0) - x) / (np.sqrt(np.sum(ce ** 2, axis=0)) / nc))
        if nc >= 8:
            zs.append(np.abs(ca.mean(0) - x) / (ca.std(0, ddof=1) / np.sqrt(nc)))
    z = np.concatenate(z)
    zs = np.concatenate(zs) if zs else np.zeros(0)
    outer = float(np.dot(nmcs, chains))
    burn = 500.0 * sum(chains)
    t = float(np.mean(ms)) * 1e-3
    return {"metric": "integrals/s (C3: 4,096 uneven integrals, ndim 1-64, MultiStepMove)", "value": args.integrals / t,
            "unit": "integrals/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": "C3 uneven batch", "integrals": args.integrals,
                       "samples_per_integral": "2^U(14,20), split over ceil(NMC / 16384) chains",
                       "chains": int(sum(chains)), "outer_steps": outer, "burnin_steps": burn, "sub_moves": 4,
                       "launch": "one persistent launch + estimators + read-back in one CUDA graph",
                       "tuning": {"threads_per_block": block, "unroll_per_ndim_bucket": unroll},
                       "calibration": "off (sub-chain on the full target: every outer step accepted)",
                       "l2": "working set (walkers in shared memory, block sums) below L2; no flush"},
            "outer_steps_per_s": (outer + burn) / t,
            "e2e": {"value": args.integrals / float(np.mean(wall)), "unit": "integrals/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": int(2 * 8 * sum(len(x) * c for x, c in zip(exact, chains)))},
            "accuracy": {"block_moments_within_3_sigma": float(np.mean(z < 3.0)), "max_z": float(z.max()),
                         "sigma": "block errors of the chains",
                         "within_3_sigma_spread_8plus_chains": float(np.mean(zs < 3.0)) if zs.size else None,
                         "max_z_spread_8plus_chains": float(zs.max()) if zs.size else None},
            "clocks": ck}


C4_NDIM, C4_NCOMP = 32, 8


def c4_target(seed=404):
    rng = np.random.default_rng(seed)
    means = rng.standard_normal((C4_NCOMP, C4_NDIM)) * 3.0
    widths = 10.0 ** rng.uniform(np.log10(0.3), np.log10(3.0), (C4_NCOMP, C4_NDIM))
    w = rng.dirichlet(np.ones(C4_NCOMP))
    params = np.concatenate([[C4_NCOMP], w, means.ravel(), widths.ravel()])
    m1 = (w[:, None] * means).sum(0)
    m2 = (w[:, None] * (widths ** 2 + means ** 2)).sum(0)
    return params, w, means, widths, m1, m2


def run_c4(args):
    """Precision study: 32-D mixture of 8 anisotropic Gaussians, 16,384 chains x 65,536 steps,
    observables x.x, x_i, x_i^2 in 64-block BlockAccumulators.  Float walker on 8 lanes per
    chain (mcig_lanes.cuh) with the Metropolis decision certified in double near the float
    threshold; Kahan float block sums against double block sums (identical trajectories),
    and the one-lane kernel for comparison.  The FP64 oracle (reference formula, double
    walker) runs 64 of the chains from the device's burnt-in state on the same Philox draws:
    the error of the float result against FP64, and the CPU leg (oracle steps/s on the host
    threads).  Metric: walker steps/s of the Kahan-float run."""
    import mcintegratorplusplus_gb300 as mcig
    params, w, means, widths, m1, m2 = c4_target()
    nch, nmc = args.chains4, args.nmc4
    rng = np.random.default_rng(1)
    comp = rng.choice(C4_NCOMP, nch, p=w)
    x0 = means[comp] + widths[comp] * rng.standard_normal((nch, C4_NDIM))
    exact = np.concatenate([[m2.sum()], m1, m2])
    out = {}
    runs = (("f32_kahan", mcig.PREC_FP32, 8), ("f64_sums", mcig.PREC_FP32_ACC64, 8), ("one_lane_kahan", mcig.PREC_FP32, 0))
    clocks = Clocks()
    clocks.start()
    for name, prec, lanes in runs:
        m = mcig.MCI(C4_NDIM, nch, precision=prec)
        m.setSeed(31)
        m.addSamplingFunction(mcig.PDF_GAUSS_MIX, params)
        m.setTrialMove(mcig.MOVE_ALL, mcig.SRRD_GAUSSIAN)
        m.setNdecorrelationSteps(256)
        bs = nmc // 64
        for kind in (mcig.OBS_X2SUM, mcig.OBS_XND, mcig.OBS_X2):
            m.addObservable(kind, (), bs, 1, False, mcig.EST_UNCORRELATED)
        if lanes:
            m.setLanes(lanes)
            m.setFP64Decision(1)
        ms, phases = [], {}
        for it in range(args.warmup + args.steps):
            m.setX(x0)
            m.integrate(0, True, True)  # calibration and burn-in
            t0 = m.getLastTimings()
            state = (m.getX(), m.getMRT2Steps(), m.getStepCounters())
            avg, err = m.integrate(nmc, False, False)
            t1 = m.getLastTimings()
            if it >= args.warmup:
                ms.append(_timed_device_ms(t0) + _timed_device_ms(t1))
                phases = {"calibration_ms": t0["calibration_ms"], "burnin_ms": t0["burnin_ms"],
                          "sampling_ms": t1["sampling_ms"], "estimation_ms": t1["estimation_ms"]}
        data = np.concatenate([m.getObsData(o) for o in range(3)], axis=1)
        ca, _ = m.getChainResults()
        stats = m.getDecisionStats() if lanes else None
        out[name] = {"ms": float(np.mean(ms)), "avg": avg, "err": err, "data": data, "ca": ca, "phases": phases,
                     "state": state, "stats": stats}
    ck = clocks.stop()
    t_k = out["f32_kahan"]["ms"] * 1e-3
    dk, dd = out["f32_kahan"]["data"], out["f64_sums"]["data"]
    rel = np.abs(dk - dd) / np.maximum(np.abs(dd), 1e-3)
    zs = {}
    for name in out:
        ca = out[name]["ca"]
        sem = ca.std(0, ddof=1) / np.sqrt(nch)
        zs[name] = float(np.max(np.abs(ca.mean(0) - exact) / sem))
    line = {"metric": "walker steps/s (C4: 16,384 chains x 32-D mixture of 8, float walker, Kahan float sums)",
            "value": nch * nmc / t_k, "unit": "walker steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_k * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (Metropolis decision certified in f64 near the threshold)",
            "data": "synthetic (seeded mixture, chains start in exact samples)",
            "config": {"workload": "C4 precision study", "chains": nch, "ndim": C4_NDIM, "components": C4_NCOMP,
                       "nmc": nmc, "blocks": 64, "observables": "x.x, x_i, x_i^2", "lanes_per_chain": 8,
                       "l2": "block output below L2; no flush"},
            "f64_sums_steps_per_s": nch * nmc / (out["f64_sums"]["ms"] * 1e-3),
            "one_lane_steps_per_s": nch * nmc / (out["one_lane_kahan"]["ms"] * 1e-3),
            "phases_ms": {k: out[k]["phases"] for k in out},
            "fp64_decision": {"steps_tested_in_f64": out["f32_kahan"]["stats"][0],
                              "float_decisions_reversed": out["f32_kahan"]["stats"][1],
                              "steps": int(out["f32_kahan"]["state"][2].sum()) + nch * nmc},
            "kahan_vs_double_block_means_max_rel": float(rel.max()),
            "max_z_vs_analytic": zs, "clocks": ck}
    if args.cpu_baseline:
        line["cpu_baseline"], line["error_vs_fp64_oracle"] = c4_oracle_leg(args, out["f32_kahan"], params, nmc)
    return line


def c4_oracle_leg(args, run, params, nmc, K=64):
    """The FP64 oracle on K chains from the device's burnt-in state, on the device chains' Philox
    draws: per-chain estimates of the float run against FP64, and the oracle's walker steps/s."""
    from oracle import oracle as orc
    x, steps, ctr = run["state"]
    o = orc.OracleMCI(C4_NDIM, K)
    o.add_sampling_function(5, params)
    o.set_trial_move(0, 1, 0)
    bs = nmc // 64
    for kind in (0, 1, 2):
        o.add_observable(kind, (), bs, 1, False, 1)
    o.set_x(x[:K])
    o.set_chain_steps(steps[:K])
    o.set_philox(31, 0, ctr[:K], layout=1)
    nthreads = os.cpu_count() or 1
    t0 = time.perf_counter()
    _, _, oca, oce = o.integrate(nmc, False, False, nthreads=nthreads, per_chain=True)
    dt = time.perf_counter() - t0
    ca = run["ca"][:K]
    d = ca - oca
    sem = oca.std(0, ddof=1) / np.sqrt(K)
    cpu = {"value": K * nmc / dt, "unit": "walker steps/s", "cores": nthreads, "kind": "port",
           "sample": "%d chains x %d steps of the workload from the device's burnt-in state, %.1f s" % (K, nmc, dt)}
    err = {"chains": K, "same_draws": "Philox counters of the device chains (float draws evaluated in double)",
           "max_abs_diff_per_chain": float(np.abs(d).max()),
           "median_rel_diff_per_chain": float(np.median(np.abs(d) / np.maximum(np.abs(oca), 1.0))),
           "combined_max_abs_diff_over_sem": float(np.max(np.abs(d.mean(0)) / sem))}
    return cpu, err


C5_ADAPT = 200  # adaptation cycles (period - 1 local steps + one Adam step on all chain positions)


def c5_target(seed=2024, ndim=24):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((ndim, 2)))
    means = np.stack([3 * Q[:, 0], -3 * Q[:, 0], 3 * Q[:, 1], -3 * Q[:, 1]])
    params = np.concatenate([[4.0], np.full(4, 0.25), means.ravel(), np.ones(4 * ndim)])
    var_x1 = 1.0 + (means[:, 0] ** 2).mean()
    return params, means, var_x1


def run_c5(args):
    """Learned proposal: 24-D mixture of 4 unit Gaussians at +-3 u1, +-3 u2, 16,384 chains,
    affine-coupling flow (8 layers, hidden 128, bf16 tensor cores) proposing every 5th step,
    against plain Gaussian Metropolis on the same chains.  ESS of <x_1> from the spread of the
    chain means (ESS = Var(x_1) * chains / var(chain means), the C2 definition), with tau_int of
    x_1 from MJBlocker and Sokal's window on 256 chains' series.  Metric: ESS/s with the flow."""
    import mcintegratorplusplus_gb300 as mcig
    D, nch, nmc = 24, args.chains5, args.nmc5
    adapt = getattr(args, "c5_adapt", None) or C5_ADAPT
    lr = getattr(args, "c5_lr", None) or 3e-3
    batch = getattr(args, "c5_batch", None) or nch
    lanes = getattr(args, "c5_lanes", 0) or 0
    params, means, var_x1 = c5_target()
    res = {}
    for use_flow in (False, True):
        ms, ess, accs = [], [], []
        for it in range(args.warmup + args.steps):
            m = mcig.MCI(D, nch, precision=mcig.PREC_FP32)
            m.setSeed(77 + it)
            m.setX(np.random.default_rng(5 + it).standard_normal((nch, D)) * 3.0)
            m.addSamplingFunction(mcig.PDF_GAUSS_MIX, params)
            m.setTrialMove(mcig.MOVE_ALL, mcig.SRRD_GAUSSIAN)
            m.setNdecorrelationSteps(1000)
            m.setFullStorage(32)
            if lanes:
                m.setLanes(lanes)
            m.addObservable(mcig.OBS_XI, [0], 1, 1, False, mcig.EST_UNCORRELATED)
            if use_flow:
                f = mcig.Flow(D, 8, 128, seed=6 + it)
                f.set_tensor_path({"mma.sync": 0, "tcgen05": 1, "mma.sync-smem": 2}[getattr(args, "c5_flow_gemm", "mma.sync")])
                _, _, acc = mcig.integrate_flow(m, f, nmc, period=5, refresh=4096, train_steps=adapt,
                                                batch=batch, lr=lr)
                accs.append(acc)
            else:
                m.integrate(nmc)
            if it >= args.warmup:
                tm = m.getLastTimings()
                ms.append(_timed_device_ms(tm))
                ca, _ = m.getChainResults()
                rep = ess_report(ca[:, 0], var_x1, nch, nmc, series=m.getObsDataChains(0, 0, min(256, nch)),
                                 mj=lambda x: mcig.estimate(mcig.EST_MJBLOCKER, x))
                ess.append(rep["ess"])
        t = float(np.mean(ms)) * 1e-3
        res[use_flow] = (float(np.mean(ess)) / t, t, float(np.mean(ess)), float(np.mean(accs)) if accs else None,
                         {k: float(v) for k, v in tm.items()}, rep)
    ratio = res[True][0] / res[False][0]
    return {"metric": "effective samples/s of <x_1> (C5: 24-D 4-mode mixture, learned flow proposal)",
            "value": res[True][0], "unit": "effective samples/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": res[True][1] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 walker, bf16 flow GEMMs (f32 accumulate)", "flow_gemms": getattr(args, "c5_flow_gemm", "mma.sync"),
            "data": "synthetic (seeded mixture, random-init flow)",
            "config": {"workload": "C5 learned proposal", "chains": nch, "ndim": D, "nmc": nmc, "flow_layers": 8,
                       "hidden": 128, "period": 5, "adaptation_cycles": adapt, "adam_batch": batch,
                       "adam_lr": lr, "refresh": 4096, "local_lanes_per_chain": lanes or 1},
            "plain_mh": {"value": res[False][0], "ms_per_step": res[False][1] * 1e3, "ess": res[False][2],
                         "phases": res[False][4], "ess_detail": res[False][5]},
            "flow": {"ess": res[True][2], "acceptance": res[True][3], "phases": res[True][4],
                     "ess_detail": res[True][5]},
            "ess_per_s_ratio_flow_over_plain": ratio}


def run_c2_parts(args):
    """Cost of the parts of a C2 step: one sampling launch (65,536 chains x 1,000 steps,
    fixed step size, no calibration or burn-in) per configuration, from the bare step to the
    bench's four accumulators.  Under ncu each launch is one configuration, in this order."""
    import mcintegratorplusplus_gb300 as mcig
    Sigma, P = target()
    all4 = [(0, 100), (1, 100), (0, 1), (1, 1)]
    cases = [("gauss_move_gauss_pdf", mcig.SRRD_GAUSSIAN, "gauss", []),
             ("uniform_move_gauss_pdf", mcig.SRRD_UNIFORM, "gauss", []),
             ("gauss_move_precision_pdf", mcig.SRRD_GAUSSIAN, "prec", []),
             ("+ x.x Block", mcig.SRRD_GAUSSIAN, "prec", [(0, 100)]),
             ("+ x_i Full", mcig.SRRD_GAUSSIAN, "prec", [(1, 1)]),
             ("+ x.x, x_i Block and Full (bench)", mcig.SRRD_GAUSSIAN, "prec", all4)]
    out = []
    for name, srrd, pdf, obs in cases:
        m = mcig.MCI(NDIM, args.chains, precision=mcig.PREC_FP32)
        m.setSeed(1)
        m.addSamplingFunction(mcig.PDF_GAUSS_PREC, P) if pdf == "prec" else m.addSamplingFunction(mcig.PDF_GAUSS)
        m.setTrialMove(mcig.MOVE_ALL, srrd)
        m.setMRT2Step(0.3)
        m.setNfindMRT2Iterations(0)
        m.setNdecorrelationSteps(0)
        m.setFullStorage(32)
        for kind, bs in obs:
            m.addObservable(kind, (), bs, 1, False, mcig.EST_UNCORRELATED)
        m.integrate(1000)
        out.append({"configuration": name, "sampling_ms": float(m.getLastTimings()["sampling_ms"])})
    return {"workload": "C2 step parts", "chains": args.chains, "steps": 1000, "parts": out}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--chains", type=int, default=NCHAINS)
    ap.add_argument("--nmc", type=int, default=NMC)
    ap.add_argument("--blocks", type=int, default=NBLOCKS)
    ap.add_argument("--cpu-chains", type=int, default=32)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-learned", dest="learned", action="store_false",
                    help="skip the learned-proposal comparison added to the default line")
    ap.add_argument("--no-batched", dest="batched", action="store_false",
                    help="skip the uneven-batch (C3) figures added to the default line")
    ap.add_argument("--c2-kernel", default="auto", choices=["auto", "one-lane", "pair"],
                    help="C2 burn-in and sampling kernel: the library's choice, one lane or two lanes per chain")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c4", "c5", "c2_parts"])
    ap.add_argument("--integrals", type=int, default=4096)
    ap.add_argument("--c3-tuning", default=None,
                    help="C3 without the autotuner: 'block,u8,u16,u32,u64' (threads per block, unroll per bucket)")
    ap.add_argument("--chains4", type=int, default=16384)
    ap.add_argument("--nmc4", type=int, default=65536)
    ap.add_argument("--chains5", type=int, default=16384)
    ap.add_argument("--nmc5", type=int, default=8192)
    ap.add_argument("--c5-adapt", type=int, default=None, help="adaptation cycles of the flow (default C5_ADAPT)")
    ap.add_argument("--c5-batch", type=int, default=None, help="rows per Adam step of the flow (default: all chains)")
    ap.add_argument("--c5-lr", type=float, default=None, help="Adam learning rate of the flow (default 3e-3)")
    ap.add_argument("--c5-lanes", type=int, default=0, choices=[0, 4, 8],
                    help="lanes per chain of the local Metropolis steps in both C5 arms (0: one lane)")
    ap.add_argument("--c5-flow-gemm", default="mma.sync", choices=["tcgen05", "mma.sync", "mma.sync-smem"],
                    help="tensor-core path of the flow's passes (the backward pass is mma.sync)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.workload != "c2" and args.impl != "reference":
        if rank == 0:
            print(json.dumps({"c3": run_c3, "c4": run_c4, "c5": run_c5,
                              "c2_parts": run_c2_parts}[args.workload](args)), flush=True)
        return
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return
    if world > 1:  # replicas only: every rank runs its own chains, rank 0 reports the max-time aggregate
        args.learned = False
        args.batched = False
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
