"""VMC step throughput of the GB300 path (one JSON line on stdout).

Workload: transverse-field Ising 10x10 periodic (J=1, h=3), ConvNetAutoregressive2D
depth 10, 32 channels (weight-normalised), 4096 exact samples per step from the
persistent sampler, local energy over the 101 connected configurations of each
sample, adjoint gradient, Adam -- the full VMC step of the BF16 tensor-core path.
The same step on the plain FP32 CUDA-core path of the same code is timed beside
it. Synthetic, seeded: random-init weights, Philox samples.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the reference algorithm (the
reference is TensorFlow 1.x and cannot run here) on the host cores, on a
bounded sample of the same workload.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SHAPE = (10, 10)
DEPTH = 10
CHANNELS = 32
BATCH = 4096
H_FIELD = 3.0
METRIC = "VMC steps/s & samples/s, BF16+adjoint vs plain FP32 on GPU at matched energy"
WORKLOAD = "TFIM 10x10 PBC J=1 h=3; ConvNetAutoregressive2D depth 10 F32 (weight norm); 4096 samples/step; " \
           "full VMC step: exact AR sampling + local energy (101 conn/sample) + adjoint gradient + Adam"


def flops_per_sample_forward(shape, depth, f):
    """Dense conv FLOPs of one forward (2 * MACs/site * sites), zero-padded
    taps included: the reference's per-unit figure."""
    n_cc = 2 * depth - 2
    first = 9 * f + 3 * f + 2 * f * (f // 2) + 9 * f * f
    rest = 22 * f * f
    head = 4 * f
    return 2 * (first + (n_cc - 1) * rest + head) * shape[0] * shape[1]


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--fp32-steps", type=int, default=10)
    p.add_argument("--matched-steps", type=int, default=150,
                   help="training steps of each path in the bench line's matched-energy leg (0: skip)")
    p.add_argument("--matched-batch", type=int, default=1024)
    p.add_argument("--matched-samples", type=int, default=16384)
    p.add_argument("--cpu-samples", type=int, default=128,
                   help="samples of one VMC step per timed CPU step (reference arm and cpu_baseline)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--case", default="vmc", choices=["vmc", "forward", "energy4x4", "vmc16", "ising12", "matched",
                                                     "j1j2sr", "chain64", "kernels", "sampler"],
                   help="forward: only the batched AR2D forward of the local-energy stage on --configs "
                        "connected configurations (the small case used for ncu captures); energy4x4: train "
                        "the 4x4 Heisenberg model (depth 5, 16 channels) and compare its exact energy "
                        "(enumeration of all 2^16 states) with Lanczos, in --precision")
    p.add_argument("--precision", default="bf16", choices=["bf16", "fp16", "fp32"])
    p.add_argument("--sr-steps", type=int, default=20)
    p.add_argument("--sr-rows-bytes", type=int, default=None,
                   help="j1j2sr: stream the per-sample rows into the SR Gram through a buffer of this many bytes")
    p.add_argument("--sr-leg-steps", type=int, default=3,
                   help="timed steps per precision of the bench line's J1-J2 SR leg (0: skip)")
    p.add_argument("--precisions", nargs="+", default=None, choices=["bf16", "fp16", "fp32"])
    p.add_argument("--optimizer", default="adam", choices=["adam", "sr"])
    p.add_argument("--lr", type=float, default=0.02)
    p.add_argument("--diag-shift", type=float, default=1e-3)
    p.add_argument("--sweeps", type=int, default=2000)
    p.add_argument("--train-steps", type=int, default=24000)
    p.add_argument("--train-batch", type=int, default=2048)
    p.add_argument("--configs", type=int, default=32768)
    p.add_argument("--lattice", type=int, nargs=2, default=None)
    p.add_argument("--depth", type=int, default=None)
    p.add_argument("--channels", type=int, default=None)
    p.add_argument("--batch", type=int, default=8192)
    p.add_argument("--weights", default=None, help="ising12: a Keras weight file of the reference's 12x12 models")
    p.add_argument("--gamma", type=float, default=3.0)
    p.add_argument("--samples", type=int, default=1 << 15)
    return p.parse_args()


def forward_case(args):
    """The AR2D forward of the local-energy stage alone, on `configs`
    configurations of the bench workload's network (or of the network given
    by --lattice/--depth/--channels), in --precision."""
    from flowket_gb300.machines import ConvNetAutoregressive2D
    shape = tuple(args.lattice) if args.lattice else SHAPE
    depth, f = args.depth or DEPTH, args.channels or CHANNELS
    m = ConvNetAutoregressive2D(shape, depth, f, weights_normalization=True, precision=args.precision, seed=0)
    g = torch.Generator(device="cuda").manual_seed(0)
    spins = (2 * torch.randint(0, 2, (args.configs,) + shape, device="cuda", generator=g) - 1).to(torch.int8)
    for _ in range(args.warmup):
        m.forward(spins)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(args.steps):
        m.forward(spins)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / args.steps
    fl = flops_per_sample_forward(shape, depth, f) * args.configs
    print(json.dumps({"case": "forward", "lattice": list(shape), "depth": depth, "channels": f,
                      "precision": args.precision, "configs": args.configs, "ms_per_forward": ms,
                      "tflops": fl / (ms / 1e3) / 1e12}), flush=True)


def vmc16_case(args):
    """Heisenberg 16x16 PBC (Marshall sign), ConvNetAutoregressive2D depth 20,
    64 channels (weight norm), `--batch` samples per step: full VMC steps
    (exact sampling, local energy over the connected configurations with
    causal reuse, adjoint gradient) of the BF16 path and of the plain FP32
    path of the same code, each after one warm-up step, CUDA-event timed.
    Both start from the same seeded parameters. `--optimizer adam` (lr 1e-3)
    or `sr`: stochastic reconfiguration (diag shift 1e-3, lr 0.05, CG) with
    the per-sample rows streamed into the Gram conv by conv (their
    num_params x 2B array, 222 GB at 8192 samples, is never stored); with SR
    both paths run the same `--steps` timed steps and the peak device memory
    of each path is reported."""
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.optimization import VariationalMonteCarlo
    from flowket_gb300.optimizers import Adam, ComplexValuesStochasticReconfiguration
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape = (16, 16)
    sr = args.optimizer == "sr"
    out = {"case": "vmc16", "workload": "Heisenberg 16x16 PBC, Marshall sign; ConvNetAutoregressive2D depth 20 F64 "
                                        "(weight norm); full VMC step with " +
                                        ("SR (diag shift 1e-3, lr 0.05, streamed Gram)" if sr else "Adam"),
           "batch": args.batch}
    for prec in args.precisions or ["bf16", "fp32"]:
        m = ConvNetAutoregressive2D(shape, 20, 64, weights_normalization=True, precision=prec, seed=0)
        vmc = VariationalMonteCarlo(m, Heisenberg(hilbert_state_shape=shape, pbc=True),
                                    FastAutoregressiveSampler(m, args.batch, seed=1234))
        if sr:
            opt = ComplexValuesStochasticReconfiguration(m, lr=0.05, diag_shift=1e-3)
        else:
            opt = Adam(m, lr=1e-3)
        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats()
        vmc.step(opt)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        steps = max(1, args.steps if (prec == "bf16" or sr) else args.fp32_steps)
        torch.cuda.synchronize()
        a.record()
        for _ in range(steps):
            vmc.step(opt)
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / steps
        out[prec] = {"ms_per_step": ms, "samples_per_s": args.batch / (ms / 1e3), "steps": steps,
                     "stage_ms": vmc.times, "energy": vmc.current_energy.real,
                     "peak_memory_gb": torch.cuda.max_memory_allocated() / 1e9}
        if sr:
            out[prec].update({"num_params": m.num_params, "streamed": opt.streamed,
                              "cg_iterations_last": float(opt.last_stats[0]),
                              "per_sample_rows_gb_if_stored": 2 * m.num_params * args.batch * 4 / 1e9})
        del vmc, opt, m
        torch.cuda.empty_cache()
    if "bf16" in out and "fp32" in out:
        out["bf16_over_fp32"] = out["fp32"]["ms_per_step"] / out["bf16"]["ms_per_step"]
    print(json.dumps(out), flush=True)


def train_and_evaluate(precision, steps, batch, eval_samples, lr=1e-3):
    """The bench workload (TFIM 10x10 PBC h=3, depth 10, 32 channels, weight
    norm) trained from the seeded initial parameters for `steps` VMC steps of
    `batch` samples with Adam on one path, then its energy estimated from
    `eval_samples` fresh samples of its own sampler: energy, standard error,
    local-energy variance, training time and throughput."""
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.observables import Observable, energy_stats
    from flowket_gb300.operators import Ising
    from flowket_gb300.optimization import VariationalMonteCarlo
    from flowket_gb300.optimizers import Adam
    from flowket_gb300.samplers import FastAutoregressiveSampler
    op = Ising(h=H_FIELD, hilbert_state_shape=SHAPE, pbc=True)
    m = ConvNetAutoregressive2D(SHAPE, DEPTH, CHANNELS, weights_normalization=True, precision=precision, seed=0)
    vmc = VariationalMonteCarlo(m, op, FastAutoregressiveSampler(m, batch, seed=1234))
    opt = Adam(m, lr=lr)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        vmc.step(opt, sync=False)
    b.record()
    torch.cuda.synchronize()
    if steps:
        vmc.finish_step()
    train_ms = a.elapsed_time(b)
    sampler = FastAutoregressiveSampler(m, min(eval_samples, 8192), seed=777)
    obs = Observable(op)
    loc = []
    for _ in range(max(1, eval_samples // sampler.batch_size)):
        spins, lp, saved = sampler.sample()
        loc.append(obs.local_values(m, spins, log_psi=lp, base_saved=saved).clone())
    stats, _ = energy_stats(torch.cat(loc))
    st = stats.tolist()
    n = sum(x.shape[0] for x in loc)
    return {"energy": st[0], "stderr": math.sqrt(st[2] / n), "local_energy_variance": st[2], "eval_samples": n,
            "train_steps": steps, "train_ms": train_ms,
            "train_samples_per_s": steps * batch / (train_ms / 1e3) if steps else None}


def matched_summary(steps, batch, eval_samples):
    out = {"train_steps": steps, "batch": batch, "eval_samples": eval_samples, "optimizer": "Adam lr 1e-3",
           "init": "same seeded parameters and sampler seed for both paths"}
    for prec in ("bf16", "fp16", "fp32"):
        out[prec] = train_and_evaluate(prec, steps, batch, eval_samples)
    e32 = out["fp32"]["energy"]
    for prec in ("bf16", "fp16"):
        e = out[prec]["energy"]
        out[prec]["relative_difference_to_fp32"] = abs(e - e32) / abs(e32)
        out[prec]["difference_in_stderr"] = abs(e - e32) / math.hypot(out[prec]["stderr"], out["fp32"]["stderr"])
        out[prec]["variance_ratio_to_fp32"] = out[prec]["local_energy_variance"] / out["fp32"]["local_energy_variance"]
        out[prec]["speedup_over_fp32"] = out[prec]["train_samples_per_s"] / out["fp32"]["train_samples_per_s"]
    out["relative_difference"] = out["bf16"]["relative_difference_to_fp32"]
    out["bf16_over_fp32"] = out["bf16"]["speedup_over_fp32"]
    return out


def matched_case(args):
    """The metric's "at matched energy" at a chosen length: both paths trained
    from the same seeded parameters for `--train-steps` VMC steps of `--batch`
    samples, energies from `--samples` fresh samples each."""
    out = {"case": "matched", "workload": WORKLOAD}
    out.update(matched_summary(args.train_steps, args.batch, args.samples))
    print(json.dumps(out), flush=True)


def j1j2sr_summary(steps, precisions, rows_bytes=None):
    """J1-J2 10x10 periodic, J2/J1 = 0.5 (operators/j1j2.py edge list);
    ConvNetAutoregressive2D depth 20, 32 channels (weight norm), Re and Im
    heads; 1024 exact samples per step; stochastic reconfiguration
    (diag_shift 1e-3, lr 0.05; Gram on the tensor cores for BF16/FP16, on the
    CUDA cores for the plain FP32 path; FP64 CG). Runs `steps` full steps
    (sampling, local energy over the used connections, per-sample
    log-derivatives, Gram, solve, update) on each precision from the same
    seeded parameters after one untimed step: ms per step, stage split,
    energy and variance per step. With `rows_bytes` the per-sample rows are
    streamed into the Gram through a buffer of that size instead of stored."""
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.operators import J1J2
    from flowket_gb300.optimization import VariationalMonteCarlo
    from flowket_gb300.optimizers import ComplexValuesStochasticReconfiguration
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape, b = (10, 10), 1024
    op = J1J2(hilbert_state_shape=shape, j2=0.5, pbc=True)
    out = {"workload": "J1-J2 10x10 PBC J2=0.5; ConvNetAutoregressive2D depth 20 F32 (weight norm); 1024 "
                       "samples/step; full VMC step with SR diag_shift 1e-3 lr 0.05", "steps": steps}
    for prec in precisions:
        m = ConvNetAutoregressive2D(shape, 20, 32, weights_normalization=True, precision=prec, seed=0)
        vmc = VariationalMonteCarlo(m, op, FastAutoregressiveSampler(m, b, seed=1234))
        opt = ComplexValuesStochasticReconfiguration(m, lr=0.05, diag_shift=1e-3, rows_bytes=rows_bytes)
        vmc.step(opt)
        energies, variances, ms, stages = [], [], [], []
        for _ in range(steps):
            a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            vmc.step(opt)
            e.record()
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(e))
            stages.append(vmc.times)
            energies.append(vmc.current_energy.real)
            variances.append(vmc.current_local_energy_variance)
        out[prec] = {"ms_per_step": float(np.mean(ms)), "steps_per_s": 1e3 / float(np.mean(ms)),
                     "samples_per_s": b / (float(np.mean(ms)) / 1e3),
                     "stage_ms": {k: float(np.mean([st[k] for st in stages])) for k in stages[0]},
                     "energy_first": energies[0], "energy_last": energies[-1], "energies": energies,
                     "variance_last": variances[-1], "cg_iterations_last": float(opt.last_stats[0].item()),
                     "num_params": m.num_params, "rows_streamed": opt.streamed}
        del m, vmc, opt
        torch.cuda.empty_cache()
    for prec in ("bf16", "fp16"):
        if prec in out and "fp32" in out:
            out[prec + "_over_fp32"] = out["fp32"]["ms_per_step"] / out[prec]["ms_per_step"]
    return out


def j1j2sr_case(args):
    out = {"case": "j1j2sr"}
    out.update(j1j2sr_summary(args.sr_steps, args.precisions or ["bf16", "fp16", "fp32"], args.sr_rows_bytes))
    print(json.dumps(out), flush=True)


def chain64_case(args):
    """Heisenberg chain L=64 periodic (Marshall sign); RBM alpha=4 with
    complex weights N(0, 0.01); 256 Metropolis-Hastings chains with local
    exchange moves, `--sweeps` sweeps per chain (one proposal per chain per
    sweep, a sample recorded every 20 sweeps), the plain sampler; then the
    learned independent proposal (ConvNetAutoregressive2D on 1 x 64, depth 4,
    16 channels, BF16) fitted to the plain chains' samples by maximum
    likelihood with the project's forward, adjoint and Adam kernels, run for
    the same number of recorded samples with the exact |psi|^2 q ratio
    acceptance. Reports each sampler's energy, its error bar with the
    integrated autocorrelation time (metropolis_hastings.py:67-89), the
    acceptance ratio and the time."""
    from flowket_gb300.machines import RBM, ConvNetAutoregressive2D
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.samplers import (MetropolisHastingsExchange, MetropolisHastingsIndependent,
                                        r_hat_and_correlations)
    L, chains, every = 64, 256, 20
    spc = max(2, args.sweeps // every)
    op = Heisenberg(hilbert_state_shape=(L,), pbc=True)
    m = RBM((L,), alpha=4, stddev=0.01, seed=0)
    out = {"case": "chain64", "workload": "Heisenberg chain L=64 PBC; RBM alpha=4 complex N(0, 0.01); 256 chains",
           "sweeps_per_chain": spc * every, "samples_per_chain": spc}

    def summary(samples, seconds, acc):
        e = m.local_energy(op, samples)[:, 0]
        r_hat, var, cs, ess = r_hat_and_correlations(e, chains)
        tau = 1 + 2 * cs
        mean = float(e.mean())
        return {"energy": mean, "stderr_iat": math.sqrt(var * tau / e.numel()), "tau_int": tau, "r_hat": r_hat,
                "ess": ess, "acceptance": acc, "seconds": seconds}

    plain = MetropolisHastingsExchange(m, chains * spc, num_of_chains=chains, unused_sampels=every - 1,
                                       discard_ratio=5, seed=7)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain_samples = next(plain)
    torch.cuda.synchronize()
    out["plain"] = summary(plain_samples, time.perf_counter() - t0, plain.update_acceptance_ratio())
    q = ConvNetAutoregressive2D((1, L), 4, 16, weights_normalization=True, precision="bf16", seed=8)
    ind = MetropolisHastingsIndependent(m, q, chains * spc, chains, seed=9, init_chains=plain.sample.clone())
    t0 = time.perf_counter()
    ind.fit_proposal(plain_samples, steps=400, lr=3e-3, batch=4096)
    torch.cuda.synchronize()
    fit_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    ind_samples = next(ind)
    torch.cuda.synchronize()
    out["learned"] = summary(ind_samples, time.perf_counter() - t0, ind.update_acceptance_ratio())
    out["learned"]["fit_seconds"] = fit_s
    out["learned"]["mean_log_likelihood"] = ind.mean_log_likelihood(plain_samples)
    d = abs(out["plain"]["energy"] - out["learned"]["energy"])
    out["energy_difference_in_sigma"] = d / math.hypot(out["plain"]["stderr_iat"], out["learned"]["stderr_iat"])
    out["tau_ratio_learned_over_plain"] = out["learned"]["tau_int"] / out["plain"]["tau_int"]
    print(json.dumps(out), flush=True)


def sampler_case(args):
    """The exact sampler of the bench network (10x10, depth 10, 32 channels,
    weight norm) at batch sizes from 1,024 to 19,456 samples (one persistent
    CTA per 128 samples: 8 to 152 CTAs on the 152 SMs), and of the 16x16
    depth-20 F64 network at 8,192: CUDA-event time per draw (best of
    `--steps` after `--warmup`) in BF16, FP16 and FP32. A draw's time that
    does not grow with the CTA count while CTAs < SMs is set by the length of
    one CTA's chain of dependent site ops, not by how many SMs work."""
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.samplers import FastAutoregressiveSampler
    out = {"case": "sampler", "network": "10x10 depth 10 F32 (weight norm)", "ms_per_draw": {}}

    def time_draw(m, b):
        smp = FastAutoregressiveSampler(m, b, seed=5)
        for _ in range(max(1, args.warmup)):
            smp.sample()
        best = float("inf")
        for _ in range(max(1, args.steps)):
            a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            smp.sample()
            e.record()
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(e))
        return best

    for prec in ("bf16", "fp16", "fp32"):
        m = ConvNetAutoregressive2D((10, 10), 10, 32, weights_normalization=True, precision=prec, seed=0)
        out["ms_per_draw"][prec] = {str(b): time_draw(m, b) for b in (1024, 2048, 4096, 8192, 16384, 19456)}
    m = ConvNetAutoregressive2D((16, 16), 20, 64, weights_normalization=True, precision="bf16", seed=0)
    out["ms_per_draw_16x16_d20_f64_bf16"] = {"8192": time_draw(m, 8192)}
    print(json.dumps(out), flush=True)


def kernels_case(args):
    """The memory-bound and FP64 kernels of the path on their own, sized
    beyond L2 (129 MB) where the kernel streams: CUDA-event time per launch
    (best of `--steps` after `--warmup`), algorithmic bytes (or FLOPs) per
    launch and the fraction of the measured HBM copy bandwidth (or of the
    cuBLAS SGEMM rate for the FP32 Gram). The small case of the per-kernel
    ncu captures."""
    from flowket_gb300 import _lib
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.observables import Observable, energy_stats
    from flowket_gb300.operators import Heisenberg, Ising
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs") or 6800.0
    g = torch.Generator(device="cuda").manual_seed(0)
    st = _lib.stream_ptr()
    out = {"case": "kernels", "hbm_peak_gbs": hbm}

    def timed(fn):
        for _ in range(max(1, args.warmup)):
            fn()
        best = float("inf")
        for _ in range(max(1, args.steps)):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            best = min(best, a.elapsed_time(b))
        return best

    def record(name, ms, nbytes=None, flops=None, peak=None, unit=None, **kw):
        r = {"ms": ms, **kw}
        if nbytes is not None:
            r.update(bytes=nbytes, gbs=nbytes / (ms / 1e3) / 1e9, frac_hbm=nbytes / (ms / 1e3) / 1e9 / hbm)
        if flops is not None:
            r.update(flops=flops, tflops=flops / (ms / 1e3) / 1e12)
            if peak:
                r.update(frac=flops / (ms / 1e3) / 1e12 / peak, peak=peak, peak_unit=unit)
        out[name] = r

    # enumeration: Ising 10x10 (101 slots) and Heisenberg 16x16 (513 slots)
    for name, op, shape, b in (("enum_ising_10x10", Ising(h=3.0, hilbert_state_shape=(10, 10), pbc=True), (10, 10),
                                1 << 18),
                               ("enum_heisenberg_16x16", Heisenberg(hilbert_state_shape=(16, 16), pbc=True),
                                (16, 16), 1 << 16)):
        spins = (2 * torch.randint(0, 2, (b,) + shape, device="cuda", generator=g) - 1).to(torch.int8)
        flat = spins.view(b, -1)
        c = op.max_number_of_local_connections
        flips = torch.empty((c, b, 2), dtype=torch.int16, device="cuda")
        mel = torch.empty((c, b), dtype=torch.float64, device="cuda")
        use = torch.empty((c, b), dtype=torch.uint8, device="cuda")
        ms = timed(lambda: op._launch(flat, b, flips, mel, use, None))
        record(name, ms, nbytes=b * (flat.shape[1] + c * 13), samples=b, slots=c)
        if name.startswith("enum_heisenberg"):
            max_rows = b * (c - 1)
            bf = {"owner": torch.empty(max_rows, dtype=torch.int32, device="cuda"),
                  "cmel": torch.empty(max_rows, dtype=torch.float64, device="cuda"),
                  "cflips": torch.empty((max_rows, 2), dtype=torch.int16, device="cuda"),
                  "offsets": torch.empty(b + 1, dtype=torch.int64, device="cuda"),
                  "nrows": torch.empty(1, dtype=torch.int64, device="cuda"),
                  "ws": torch.empty(_lib.load().fk_compact_workspace_bytes(b), dtype=torch.uint8, device="cuda")}

            def compact():
                _lib.call("fk_compact_connections", _lib.ptr(flat), b, flat.shape[1], c, _lib.ptr(flips),
                          _lib.ptr(mel), _lib.ptr(use), 1, None, _lib.ptr(bf["owner"]), _lib.ptr(bf["cmel"]),
                          _lib.ptr(bf["cflips"]), _lib.ptr(bf["offsets"]), b * (c - 1), _lib.ptr(bf["nrows"]),
                          _lib.ptr(bf["ws"]), bf["ws"].numel(), st)
            ms = timed(compact)
            rows = int(bf["nrows"].item())
            record("compact_heisenberg_16x16", ms, nbytes=b * c * 13 + rows * (4 + 8 + 4) + (b + 1) * 8, rows=rows)
    # local-energy reduction: 2^18 samples x 100 rows
    b, per = 1 << 18, 100
    rows = b * per
    lp_self = torch.randn((b, 2), device="cuda", generator=g) * 0.1 - 30.0
    lp_rows = torch.randn((rows, 2), device="cuda", generator=g) * 0.1 - 30.0
    mel0 = torch.randn(b, device="cuda", dtype=torch.float64, generator=g)
    cmel = torch.full((rows,), -3.0, device="cuda", dtype=torch.float64)
    offsets = torch.arange(0, rows + 1, per, device="cuda", dtype=torch.int64)
    local = torch.empty((b, 2), device="cuda", dtype=torch.float64)
    ms = timed(lambda: _lib.call("fk_local_energy_reduce", _lib.ptr(lp_self), _lib.ptr(mel0), b, _lib.ptr(lp_rows),
                                 _lib.ptr(offsets), _lib.ptr(cmel), _lib.ptr(local), st))
    record("local_energy_reduce", ms, nbytes=b * (8 + 8 + 8 + 16) + rows * 16, samples=b, rows=rows)
    ms = timed(lambda: energy_stats(local))
    record("energy_stats", ms, nbytes=b * (16 + 16 + 8), samples=b)
    del lp_rows, cmel
    # SR: sample-space Gram (FP32 products, FP64 reduction), FP64 CG, back-map
    p, bs = 200_000, 1024
    n = 2 * bs
    o_re = torch.randn((p, bs), device="cuda", generator=g)
    o_im = torch.randn((p, bs), device="cuda", generator=g)
    gram = torch.empty((n, n), device="cuda", dtype=torch.float64)
    ms = timed(lambda: _lib.call("fk_sr_gram", _lib.ptr(o_re), _lib.ptr(o_im), p, bs, _lib.ptr(gram), n * n, st))
    peak32 = fp32_peak_tflops()
    record("sr_gram", ms, flops=float(n) * (n + 1) * p, peak=peak32, unit="TFLOP/s (cuBLAS SGEMM, measured)",
           nbytes=2 * p * bs * 4, params=p, samples=bs)
    ms = timed(lambda: _lib.call("fk_sr_gram_tc", _lib.ptr(o_re), _lib.ptr(o_im), p, bs, _lib.ptr(gram), n * n,
                                 st))
    record("sr_gram_tc", ms, flops=float(n) * (n + 1) * p, peak=peaks.get("bf16_tflops"),
           unit="TFLOP/s (bf16 burst, measured; each product costs three bf16 MMAs)", nbytes=2 * p * bs * 4,
           params=p, samples=bs)
    sbytes = _lib.load().fk_sr_gram_split_bytes(p, n)
    split = torch.empty(sbytes, dtype=torch.uint8, device="cuda")
    ms = timed(lambda: _lib.call("fk_sr_gram_split", _lib.ptr(o_re), _lib.ptr(o_im), bs, bs, p, n, _lib.ptr(split),
                                 sbytes, st))
    record("sr_gram_split", ms, nbytes=2 * p * bs * 4 + sbytes, params=p, samples=bs,
           note="read the FP32 rows once, write bf16 hi + lo in the blocked operand layout")
    ms = timed(lambda: _lib.call("fk_sr_gram_split_accumulate", _lib.ptr(split), p, n, _lib.ptr(gram), st))
    record("sr_gram_split_accumulate", ms, flops=float(n) * (n + 1) * p, peak=peaks.get("bf16_tflops"),
           unit="TFLOP/s (bf16 burst, measured; each product costs three bf16 MMAs)", nbytes=sbytes, params=p,
           samples=bs)
    del split
    rhs = torch.randn(n, device="cuda", dtype=torch.float64, generator=g)
    alpha = torch.empty(n, device="cuda", dtype=torch.float64)
    stats = torch.zeros(3, device="cuda", dtype=torch.float64)
    ws = torch.empty(_lib.load().fk_sr_solve_workspace_bytes(n), dtype=torch.uint8, device="cuda")
    iters = 50
    ms = timed(lambda: _lib.call("fk_sr_solve", _lib.ptr(gram), n, 1.0 / bs, 1e3, _lib.ptr(rhs), 1e-30, iters,
                                 _lib.ptr(alpha), _lib.ptr(stats), _lib.ptr(ws), ws.numel(), st))
    record("sr_cg_50_iterations", ms, nbytes=iters * n * n * 8, n=n,
           note="the Gram (33.6 MB) stays in L2 across iterations: bytes are per-iteration reads")
    ms = timed(lambda: _lib.call("fk_center_columns", _lib.ptr(o_re), p, bs, None, st))
    record("sr_center_columns", ms, nbytes=2 * p * bs * 4, params=p, samples=bs,
           note="one read for the mean, one read-modify-write pass (the second read hits L2 per row)")
    x = torch.empty(p, device="cuda")
    ms = timed(lambda: _lib.call("fk_sr_backmap", _lib.ptr(o_re), _lib.ptr(o_im), p, bs, _lib.ptr(alpha), 1.0 / bs,
                                 0.0, None, _lib.ptr(x), st))
    record("sr_backmap", ms, nbytes=2 * p * bs * 4 + p * 4, params=p)
    del o_re, o_im, gram
    torch.cuda.empty_cache()
    # adjoint (tensor cores) and causal-reuse forward of the bench network
    m = ConvNetAutoregressive2D(SHAPE, DEPTH, CHANNELS, weights_normalization=True, precision=args.precision, seed=0)
    b = 4096
    spins = (2 * torch.randint(0, 2, (b,) + SHAPE, device="cuda", generator=g) - 1).to(torch.int8)
    _, _, saved = m.forward(spins, mode=_lib.FK_AR2D_SAVE)
    w = torch.randn((b, 2), device="cuda", generator=g) / b
    ms = timed(lambda: m.backward(spins, w, saved))
    fps = flops_per_sample_forward(SHAPE, DEPTH, CHANNELS)
    record("adjoint_10x10_d10_f32", ms, flops=2.0 * fps * b, peak=peaks.get("bf16_tflops_sustained"),
           unit="TFLOP/s (bf16, measured)", samples=b, note="algorithmic FLOPs: 2x the forward's")
    # per-sample rows (Re and Im log-derivatives) of 1024 samples: two
    # per-sample adjoints, the weight gradients on tcgen05 (wgrad_rows_tc_kernel)
    bo = 1024
    ms = timed(lambda: m.log_derivatives(spins[:bo], None))
    record("per_sample_rows_10x10_d10_f32", ms, nbytes=2 * m.num_params * bo * 4, samples=bo, params=m.num_params,
           note="bytes: the rows written (forward and data gradients included in the time)")
    obs = Observable(Ising(h=H_FIELD, hilbert_state_shape=SHAPE, pbc=True))
    lp, _, _ = m.forward(spins)
    ms = timed(lambda: obs.local_values(m, spins, log_psi=lp, base_saved=saved))
    record("local_energy_10x10_d10_f32_causal_reuse", ms, samples=b, rows=b * 100)
    print(json.dumps(out), flush=True)


# experiments/README.md, "Ising (2^15 sampels)": 12x12 open-boundary transverse
# Ising at field gamma, the published depth-10 32-channel models evaluated
# with the D4 x spin-flip ensemble: energy, local-energy variance, |Mz|.
PUBLISHED_ISING_12X12 = {2.0: (-346.9817926, 0.00125, 0.783929189), 2.5: (-395.6618438, 0.00421, 0.57235633),
                         3.0: (-457.0420317, 0.000821, 0.1622390747), 3.5: (-524.5172088, 0.000647, 0.1106881036),
                         4.0: (-593.5389339, 0.000777, 0.09679073758)}


def ising12_case(args):
    """The reference's published evaluation (experiments/run_evaluation.py:12-24)
    on this stack: the Keras weight file loaded into ConvNetAutoregressive2D
    (12x12, depth 10, 32 channels, weight norm), wrapped in
    make_up_down_invariant(make_2d_obc_invariants(model)), samples of the base
    model's exact sampler, local energies of the ensemble for the open-boundary
    Ising operator at field gamma; mean energy, variance and |Mz| over
    `--samples` samples, next to the published numbers."""
    from flowket_gb300.ensemble import make_2d_obc_invariants, make_up_down_invariant
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.operators import Ising
    from flowket_gb300.optimization import VariationalMonteCarlo
    from flowket_gb300.samplers import FastAutoregressiveSampler
    if not args.weights:
        raise SystemExit("--weights is required for --case ising12")
    shape = (12, 12)
    m = ConvNetAutoregressive2D(shape, 10, 32, weights_normalization=True, precision=args.precision, seed=0)
    m.load_weights(args.weights)
    ens = make_up_down_invariant(make_2d_obc_invariants(m))
    batch = min(args.batch, args.samples)
    vmc = VariationalMonteCarlo(ens, Ising(h=args.gamma, hilbert_state_shape=shape, pbc=False),
                                FastAutoregressiveSampler(m, batch, seed=2024))
    loc, mz = [], []
    t0 = time.perf_counter()
    for _ in range(max(1, args.samples // batch)):
        spins, _ = vmc.next_batch()
        loc.append(vmc.current_local_energy.real.double())
        mz.append(spins.reshape(batch, -1).double().mean(dim=1).abs())
    torch.cuda.synchronize()
    e = torch.cat(loc)
    n = e.numel()
    energy, var = float(e.mean()), float(e.var(unbiased=False))
    out = {"case": "ising12", "gamma": args.gamma, "precision": args.precision, "samples": n,
           "energy": energy, "energy_per_spin": energy / 144, "local_energy_variance": var,
           "abs_mz": float(torch.cat(mz).mean()), "stderr": math.sqrt(var / n), "seconds": time.perf_counter() - t0}
    if args.gamma in PUBLISHED_ISING_12X12:
        pe, pv, pm = PUBLISHED_ISING_12X12[args.gamma]
        out["published"] = {"energy": pe, "local_energy_variance": pv, "abs_mz": pm}
        out["energy_minus_published"] = energy - pe
    print(json.dumps(out), flush=True)


# FP64 Lanczos ground-state energy of the 4x4 periodic Heisenberg operator
# (Pauli matrices, J = 1) over the full 2^16 space; tests/test_oracle.py pins
# the oracle's Lanczos to this value.
HEISENBERG_4X4_PBC_E0 = -44.91393283371548


def energy4x4_case(args):
    """Heisenberg 4x4 PBC (Marshall sign), ConvNetAutoregressive2D depth 5,
    16 channels, no weight norm: Adam with a cosine learning-rate decay from
    1e-3 to 1e-5, exact sampling; the trained model's energy is evaluated
    exactly over all 2^16 configurations and compared with the FP64 Lanczos
    ground-state energy of the same operator."""
    import math
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.observables import Observable
    from flowket_gb300.operators import Heisenberg
    from flowket_gb300.optimization import VariationalMonteCarlo
    from flowket_gb300.optimizers import Adam
    from flowket_gb300.samplers import FastAutoregressiveSampler
    shape = (4, 4)
    op = Heisenberg(hilbert_state_shape=shape, pbc=True)
    e0 = HEISENBERG_4X4_PBC_E0
    idx = torch.arange(2 ** 16, device="cuda")
    states = (2 * ((idx[:, None] >> torch.arange(16, device="cuda")[None, :]) & 1) - 1).to(torch.int8).view(-1, 4, 4)
    obs = Observable(op)

    def exact_energy(m):
        lp, _, _ = m.forward(states)
        p = torch.exp(2 * lp[:, 0].double())
        p = p / p.sum()
        return float((p * obs.local_values(m, states, log_psi=lp)[:, 0]).sum())

    # connected states of every state as indices into the table of all
    # states (state bit k = 1 <-> spin +1 at site k; a used slot exchanges
    # two opposite spins, i.e. toggles two bits)
    flips, mel_all, use_all, _ = op.enumerate(states)
    f64 = flips.to(torch.int64)
    toggles = torch.where(f64 >= 0, torch.ones_like(f64) << f64.clamp(min=0), torch.zeros_like(f64)).sum(-1)
    conn_idx = idx[None, :] ^ toggles

    def exact_energy_table(lp):
        """Exact energy of a wave function given on every state (FP64)."""
        lpc = torch.complex(lp[:, 0].double(), lp[:, 1].double())
        p = torch.exp(2 * lpc.real)
        p = p / p.sum()
        ratio = torch.exp(lpc[conn_idx] - lpc[None, :])
        eloc = (mel_all * use_all.double() * ratio).sum(0)
        return float((p * eloc.real).sum())

    m = ConvNetAutoregressive2D(shape, 5, 16, weights_normalization=False, precision=args.precision, seed=0)
    vmc = VariationalMonteCarlo(m, op, FastAutoregressiveSampler(m, args.train_batch, seed=1234))
    if args.optimizer == "sr":
        # stochastic reconfiguration (the reference's optimizer.py:14-183),
        # learning rate decayed with the same cosine schedule
        from flowket_gb300.optimizers import ComplexValuesStochasticReconfiguration
        opt = ComplexValuesStochasticReconfiguration(m, lr=args.lr, diag_shift=args.diag_shift,
                                                     gram="tc" if args.train_batch % 8 == 0 else "fp32")
        lr0, lr1 = args.lr, args.lr * 1e-2
    else:
        opt = Adam(m, lr=1e-3)
        lr0, lr1 = 1e-3, 1e-5
    t0 = time.perf_counter()
    trace = []
    for k in range(1, args.train_steps + 1):
        opt.lr = lr1 + 0.5 * (lr0 - lr1) * (1 + math.cos(math.pi * k / args.train_steps))
        vmc.step(opt)
        if k % max(1, args.train_steps // 10) == 0:
            trace.append((k, exact_energy(m)))
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    e = exact_energy(m)
    out = {"case": "energy4x4", "precision": args.precision, "optimizer": args.optimizer,
           "steps": args.train_steps, "batch": args.train_batch, "exact_energy": e, "lanczos": e0,
           "relative_error": abs(e - e0) / abs(e0), "train_s": train_s,
           "trace_relative_error": [(k, abs(x - e0) / abs(e0)) for k, x in trace]}
    # the trained network evaluated through the reference's symmetrised
    # ensembles (machines/ensemble.py:41-66), as its published numbers are
    # (experiments/run_evaluation.py:12-24): exact energies over all states
    from flowket_gb300.ensemble import make_pbc_invariants, make_up_down_invariant
    ens = {"plain": m, "up_down": make_up_down_invariant(m),
           "translations_d4": make_pbc_invariants(m),
           "translations_d4_up_down": make_up_down_invariant(make_pbc_invariants(m))}
    out["ensembles"] = {}
    for name, mach in ens.items():
        lp, _, _ = mach.forward(states)
        en = exact_energy_table(lp)
        out["ensembles"][name] = {"exact_energy": en, "relative_error": abs(en - e0) / abs(e0)}
    print(json.dumps(out), flush=True)


def dist_init(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
        if torch.cuda.is_available():
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="fk_bench_clocks_", suffix=".csv")
        os.close(fd)

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(torch.cuda.current_device()), "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if self.proc is None:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        lines = open(self.path).read().splitlines()
        os.unlink(self.path)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if sm:
            out = {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


# ------------------------------------------------------------------ CPU arm
def cpu_vmc_sample(batch, seed, threads):
    """One VMC step of the reference algorithm restated on the CPU (oracle),
    for `batch` samples: fast AR sampling, local energy over all connections,
    autograd gradient. Returns seconds."""
    from oracle import ar2d, operators
    from oracle.fast_sampler import FastSamplerCPU
    torch.set_num_threads(threads)
    params = ar2d.init_params(SHAPE, DEPTH, CHANNELS, True, seed=0)
    p32 = ar2d.params_to(params, torch.float32)
    t0 = time.perf_counter()
    spins = FastSamplerCPU(params, SHAPE, DEPTH, True, dtype=torch.float32).sample(batch, seed=seed, offset=0)
    conn, mel, use = operators.ising_find_conn(spins, h=H_FIELD, pbc=True)
    with torch.no_grad():
        flat = torch.as_tensor(conn.reshape((-1,) + SHAPE).astype(np.int8))
        re, im = ar2d.log_psi(p32, flat, DEPTH, True)
    lv = (re.double().numpy() + 1j * im.double().numpy()).reshape(conn.shape[0], batch)
    local = (mel * np.exp(lv - lv[0])).sum(axis=0)
    y = np.conj(local - local.mean()) / batch
    ar2d.weighted_gradient(p32, spins, DEPTH, True, 2 * y.real / batch, -2 * y.imag / batch, dtype=torch.float32)
    return time.perf_counter() - t0


def reference_arm(args, rank, world):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    batch = args.cpu_samples
    # warm-up steps only warm the thread pool and allocator: a small sample
    for i in range(args.warmup):
        cpu_vmc_sample(16, 100 + i, threads)
    times = [cpu_vmc_sample(batch, i, threads) for i in range(args.steps)]
    t = float(np.mean(times))
    value = batch / t
    line = {"metric": METRIC, "value": value, "unit": "samples/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cpu_sample": f"{batch} samples per step"},
            "cpu_baseline": {"value": value, "unit": "samples/s", "cores": threads, "kind": "port",
                             "sample": f"{batch} of the 4096 samples of one VMC step per timed step (oracle "
                                       "restatement: fast AR sampler, all 101 connections, autograd); "
                                       "warm-up steps of 16 samples"},
            "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU arm
def build_problem(precision, seed_offset):
    from flowket_gb300.machines import ConvNetAutoregressive2D
    from flowket_gb300.operators import Ising
    from flowket_gb300.optimization import VariationalMonteCarlo
    from flowket_gb300.optimizers import Adam
    from flowket_gb300.samplers import FastAutoregressiveSampler
    m = ConvNetAutoregressive2D(SHAPE, DEPTH, CHANNELS, weights_normalization=True, precision=precision, seed=0)
    vmc = VariationalMonteCarlo(m, Ising(h=H_FIELD, hilbert_state_shape=SHAPE, pbc=True),
                                FastAutoregressiveSampler(m, BATCH, seed=1234 + seed_offset))
    return m, vmc, Adam(m, lr=1e-3)


def fp32_peak_tflops(n=8192, reps=5):
    """cuBLAS SGEMM (TF32 off) throughput: the FP32 CUDA-core denominator."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        g = torch.Generator(device="cuda").manual_seed(0)
        a = torch.randn((n, n), device="cuda", generator=g)
        b = torch.randn((n, n), device="cuda", generator=g)
        c = torch.empty((n, n), device="cuda")
        for _ in range(2):
            torch.matmul(a, b, out=c)
        best = float("inf")
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b, out=c)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b, c
        return 2.0 * n ** 3 / (best / 1e3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def timed_steps(vmc, opt, k):
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fwd_ms, rows = 0.0, 0
    torch.cuda.synchronize()
    start.record()
    for _ in range(k):
        vmc.step(opt, sync=False)
        fwd_ms_i, rows_i = vmc.energy_observable.last_forward
        rows += rows_i
    stop.record()
    torch.cuda.synchronize()
    for ev in vmc.energy_observable.forward_events:
        fwd_ms += ev[0].elapsed_time(ev[1])
    vmc.energy_observable.forward_events.clear()
    vmc.finish_step()
    return start.elapsed_time(stop), fwd_ms, rows


def evaluated_row_fraction(vmc):
    """Mean fraction of lattice rows the local-energy forward evaluates per
    connected configuration: causal reuse recomputes rows >= the first
    flipped row only (rows above come from the sampled configuration's saved
    activations), so the algorithmic FLOPs of a connection are this fraction
    of a full forward's."""
    obs = vmc.energy_observable
    _, _, bf, rows = obs.connections(vmc.current_batch)
    f = bf["cflips"][:rows].to(torch.int64)
    h, w = SHAPE
    r = torch.where(f >= 0, torch.div(f, w, rounding_mode="floor"), torch.full_like(f, h))
    rk = r.min(dim=1).values
    rk = torch.where(rk >= h, torch.zeros_like(rk), rk)
    return float(((h - rk).double() / h).mean())


def ours_arm(args, rank, world):
    from flowket_gb300 import _lib
    lib = _lib.load()
    m, vmc, opt = build_problem("bf16", rank)
    obs = vmc.energy_observable
    obs.record_forward = True
    for _ in range(args.warmup):
        vmc.step(opt)
    row_frac = evaluated_row_fraction(vmc)
    obs.forward_events.clear()
    clocks = Clocks()
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    l0 = lib.fk_kernel_launches()
    total_ms, fwd_ms, rows = timed_steps(vmc, opt, args.steps)
    launches = lib.fk_kernel_launches() - l0
    clk = clocks.stop()
    barrier(world)
    total_ms = max_over_ranks(total_ms, world)
    ms_per_step = total_ms / args.steps
    samples_per_s = world * BATCH * args.steps / (total_ms / 1e3)
    energy_bf16 = vmc.current_energy.real

    # e2e: the public API with the host owning the parameters (pinned) and the
    # reference's host-side outputs (samples, local energies, energy stats).
    host_params = torch.empty(m.num_params, dtype=torch.float32, pin_memory=True)
    host_params.copy_(m.params)
    host_spins = torch.empty((BATCH,) + SHAPE, dtype=torch.int8, pin_memory=True)
    host_local = torch.empty((BATCH, 2), dtype=torch.float64, pin_memory=True)
    host_stats = torch.empty(3, dtype=torch.float64, pin_memory=True)
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        m.params.copy_(host_params, non_blocking=True)
        m.params_updated()
        stats = vmc.step(opt, sync=False)
        host_params.copy_(m.params, non_blocking=True)
        host_spins.copy_(vmc.current_batch, non_blocking=True)
        host_local.copy_(vmc._local, non_blocking=True)
        host_stats.copy_(stats, non_blocking=True)
        torch.cuda.current_stream().synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = {"value": world * BATCH * args.steps / e2e_s, "unit": "samples/s",
           "h2d_bytes_per_step": m.num_params * 4,
           "d2h_bytes_per_step": m.num_params * 4 + BATCH * SHAPE[0] * SHAPE[1] + BATCH * 16 + 24}

    # plain FP32 path of the same code
    fp32 = None
    if args.fp32_steps > 0:
        m32, vmc32, opt32 = build_problem("fp32", rank)
        vmc32.energy_observable.record_forward = True
        vmc32.step(opt32)
        vmc32.energy_observable.forward_events.clear()
        t32, fwd32_ms, rows32 = timed_steps(vmc32, opt32, args.fp32_steps)
        fp32 = {"samples_per_s": BATCH / (t32 / args.fp32_steps / 1e3), "ms_per_step": t32 / args.fp32_steps,
                "energy": vmc32.current_energy.real, "steps": args.fp32_steps, "stage_ms": vmc32.times}
        # roofline of the FP32 path's dominant kernels (the CUDA-core AR2D ops of
        # the local-energy forward) against cuBLAS SGEMM measured here
        peak32 = fp32_peak_tflops()
        ach32 = rows32 * row_frac * flops_per_sample_forward(SHAPE, DEPTH, CHANNELS) / (fwd32_ms / 1e3) / 1e12
        fp32["roofline"] = {"bound": "fp32 CUDA cores", "achieved": ach32, "peak": peak32, "unit": "TFLOP/s",
                            "frac": ach32 / peak32, "kernel": "AR2D conv ops (FP32) of the local-energy forward",
                            "peak_source": "measured in this run: cuBLAS SGEMM 8192^3, TF32 off, best of 5"}
        del m32, vmc32, opt32
        torch.cuda.empty_cache()

    matched = None
    if args.matched_steps > 0 and rank == 0:
        matched = matched_summary(args.matched_steps, args.matched_batch, args.matched_samples)
    sr_leg = None
    if args.sr_leg_steps > 0 and rank == 0:
        sr_leg = j1j2sr_summary(args.sr_leg_steps, ["bf16", "fp32"])

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("bf16_tflops_sustained") or 1700.0
    fps = flops_per_sample_forward(SHAPE, DEPTH, CHANNELS)
    achieved = rows * row_frac * fps / (fwd_ms / 1e3) / 1e12 if fwd_ms > 0 else None
    # DRAM bytes of one full forward per configuration, from an ncu capture of
    # the forward case (profiles/); the local-energy forward moves this
    # fraction (evaluated rows) per connected configuration
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "ar2d_forward_dram_traffic_10x10_d10_f32_c32768.json")
    if os.path.exists(tpath):
        traffic = json.load(open(tpath)).get("ar2d_forward_bytes_per_config")
    hbm = None
    if traffic and fwd_ms > 0:
        gbs = rows * row_frac * traffic / (fwd_ms / 1e3) / 1e9
        hbm_peak = peaks.get("hbm_gbs") or 6800.0
        hbm = {"achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
               "bytes_per_config": traffic}

    if rank == 0:
        line = {"metric": METRIC, "value": samples_per_s, "unit": "samples/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
                "vmc_steps_per_s": 1e3 / ms_per_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "bf16", "data": "synthetic (seeded init, Philox samples)",
                "config": {"workload": WORKLOAD, "batch_per_gpu": BATCH, "lattice": list(SHAPE), "depth": DEPTH,
                           "channels": CHANNELS, "parallelism": f"replicas x{world}",
                           "l2": "inputs larger than L2 (activation workspaces of several GB per step)"},
                "energy_bf16": energy_bf16, "fp32_path": fp32,
                "bf16_over_fp32": (samples_per_s / world) / fp32["samples_per_s"] if fp32 else None,
                "matched": matched,
                "sr_step_j1j2_10x10_d20": sr_leg,
                "stage_ms": vmc.times,
                "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                             "frac": achieved / peak if achieved else None,
                             "traffic": traffic * row_frac if traffic else None,
                             "traffic_unit": "DRAM bytes per evaluated connected configuration",
                             "hbm": hbm,
                             "kernel": "AR2D conv ops (V/H/C) of the local-energy forward",
                             "flops_per_config": fps, "configs_timed": rows,
                             "evaluated_row_fraction": row_frac},
                "clocks": clk, "gpu_launches": launches, "e2e": e2e}
        if not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            n = args.cpu_samples
            cpu_vmc_sample(16, 7, threads)
            t = cpu_vmc_sample(n, 0, threads)
            line["cpu_baseline"] = {"value": n / t, "unit": "samples/s", "cores": threads, "kind": "port",
                                    "sample": f"{n} samples of one VMC step (oracle restatement on the host: "
                                              "fast AR sampler, 101 connections each, autograd gradient)"}
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world = dist_init(args.gpus)
    if args.case == "forward":
        forward_case(args)
    elif args.case == "energy4x4":
        energy4x4_case(args)
    elif args.case == "vmc16":
        vmc16_case(args)
    elif args.case == "ising12":
        ising12_case(args)
    elif args.case == "matched":
        matched_case(args)
    elif args.case == "j1j2sr":
        j1j2sr_case(args)
    elif args.case == "chain64":
        chain64_case(args)
    elif args.case == "kernels":
        kernels_case(args)
    elif args.case == "sampler":
        sampler_case(args)
    elif args.impl == "reference":
        reference_arm(args, rank, world)
    else:
        ours_arm(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
