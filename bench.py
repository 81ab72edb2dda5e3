"""Benchmark: TEBD gate-layers/s at χ=256 (L=64, d=2) on GB300.

Workload (seeded, synthetic): random MPS L=64, d=2, χ0=16 (seed 2, bonds clamped like
rand(MPS)), brickwork layers of Haar-random 4×4 gates (layer ℓ from seed 3+ℓ), each gate
simple_update! with maxdim=256 and absolute cutoff 1e-12.  Layers 0–4 saturate the bulk
bonds at χ=256 (untimed); one step = one further brickwork layer (31–32 gates: centre
moves by QR, θ = G·A·B, 512×512 SVD, truncation, √S absorption) on the saturated MPS.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  ``value`` is the mixed-precision batched form: B independent
instances (initial states from seeds 2, 1002, …; the same circuit) advanced in lockstep,
each gate an FP32 Jacobi pre-pass + FP64 rotations / truncation / overlaps; the value
counts gate-layers of all instances.  ``fp64`` is the plain FP64 GPU path on one
instance; ``e2e`` runs the batched layers through the public MPS API from host arrays
(H2D of the MPS + gates, D2H of the result each step).  ``--impl reference``
times the CPU restatement of the reference algorithm (numpy/LAPACK on all host cores) on
the same workload.  N>1 runs independent replicas, one per GPU (no collective).
"""

from __future__ import annotations

import argparse
import faulthandler
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "tenet.jl_gb300"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

SAT_LAYERS = 5
# DRAM bytes per launch of the step's dominant kernels from one ncu capture (dram__bytes_read.sum
# + dram__bytes_write.sum, profiles/), by profiler class; None where not captured
# DRAM bytes per launch of the dominant kernels, from one ncu capture of the same shapes
# (16 instances, θ 512×512): k_jacobi_block_f32 (an outer round, dram__bytes_read.sum +
# dram__bytes_write.sum); the small-case capture has the headline step's shapes
DOMINANT_TRAFFIC = {"jacobi_fp32": 67.17e6 + 6.68e6}
L_SITES, CHI0, CHI_MAX, CUTOFF = 64, 16, 256, 1e-12
METRIC = "tebd_gate_layers_per_s_chi256"
UNIT = "layers/s"
CONFIG = {
    "workload": "tebd_L64_d2_chi16to256_brickwork_layer",
    "L": L_SITES,
    "d": 2,
    "chi0": CHI0,
    "chi_max": CHI_MAX,
    "cutoff": CUTOFF,
    "gates_per_layer": "32 (odd) / 31 (even)",
    "gate_order": "serpentine: odd layers left to right, even layers right to left",
    "saturation_layers_untimed": SAT_LAYERS,
    "step": "one brickwork layer on the saturated MPS",
    "seeds": {"mps": 2, "gates": "3+layer"},
}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nme, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nme)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(values, ws):
    """Each timing's maximum over the ranks (an all-reduce over the process group: gloo
    under torchrun here, the timings being host floats); the values themselves for one
    rank."""
    if ws <= 1:
        return list(values)
    import torch
    import torch.distributed as dist

    t = torch.tensor(list(values), dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def replica_throughput(ws, instances, steps, seconds):
    """Whole-job throughput of ws replicas, each advancing `instances` MPS by `steps`
    layers in `seconds` (the slowest rank's time)."""
    return ws * instances * steps / seconds


def layers_for(n):
    from tenetgb import workloads as W

    return W.tebd_layers(L_SITES, n, serpentine=True)


def flush_l2(torch, buf):
    buf.add_(1.0)


def bench_config(ws, batch):
    """The workload description both arms print (identical dicts)."""
    return dict(CONFIG, parallelism=f"replicas{ws}", batch_instances=batch,
                l2="flushed between steps (256 MB write)")


def _timed_layers(ctx, torch, stream, dev, l2buf, psi, layers, warm):
    """Apply `layers` to psi one at a time; the first `warm` untimed, the rest each timed
    with CUDA events on the library's stream, L2 flushed before each."""
    for ly in layers[:warm]:
        psi.evolve_brickwork_([ly], maxdim=CHI_MAX, threshold=CUTOFF)
    ctx.sync()
    times = []
    for ly in layers[warm:]:
        flush_l2(torch, l2buf)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        psi.evolve_brickwork_([ly], maxdim=CHI_MAX, threshold=CUTOFF)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    return times


def pipe_peaks(ctx):
    """Roofline denominators: HBM copy rate and BF16 dense rate from MEASURED_PEAKS.json
    (measured on this machine), the CUDA cores' FP32 and FP64 FMA rates measured here
    (tn_pipe_peak: a register-resident FMA loop over every SM)."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        mp = json.load(open(path))
        hbm, bf16, src = mp["hbm_gbs"], mp["bf16_tflops"], "MEASURED_PEAKS.json"
    else:
        hbm, bf16, src = 6800.0, 1900.0, "fallback (6.8 TB/s, 1.9 PFLOP/s bf16)"
    return {"hbm_gbs": hbm, "bf16_tflops": bf16, "fp32_tflops": ctx.pipe_peak("fp32"),
            "fp64_tflops": ctx.pipe_peak("fp64"),
            "source": f"HBM and BF16: {src} (measured); FP32 / FP64 CUDA-core FMA rate: measured in this run"}


# per profiled class: the pipe whose peak bounds its arithmetic
_PIPE = {"jacobi_fp32": ("fp32_tflops", "fp32_cuda_cores"), "jacobi_fp64": ("fp64_tflops", "fp64_cuda_cores"),
         "gemm_fp64": ("fp64_tflops", "fp64_cuda_cores"), "gemm_split_bf16": ("bf16_tflops", "tensor"),
         "split_prep": (None, "hbm"), "qr": ("fp64_tflops", "fp64_cuda_cores"),
         "jacobi_coop": ("fp64_tflops", "fp64_cuda_cores")}
_KERNEL = {"jacobi_fp32": "k_jacobi_block_f32 (FP32 block rounds)", "jacobi_fp64": "k_jacobi_step_reg<double>",
           "gemm_fp64": "k_gemm_cx<double>", "gemm_split_bf16": "k_gemm_oz (tcgen05 kind::f16)",
           "split_prep": "k_oz_scales + k_oz_split", "qr": "k_qr_panel + k_apply_block_reflector",
           "jacobi_coop": "k_jacobi_coop<double>"}


# what ncu shows bounds each class beyond the two roofs (profiles/ summaries)
_LIMIT = {"jacobi_fp32": "instruction issue (ncu: 56-61 % of issue slots busy, one 512-thread CTA per SM); DRAM "
                         "traffic is half the algorithmic bytes (the rest hits L2)",
          "gemm_split_bf16": "N = 64 tiles (TMEM holds 8 levels x 64 columns): tensor subpipe 64 % busy yields 0.21 "
                             "of peak; one CTA per SM, epilogue not overlapped",
          "qr": "the FP64 pipe (one panel CTA per matrix between block-reflector updates)"}


def kernel_rooflines(prof, peaks):
    """Per profiled class (event-timed inside the step): launches, ms, the algorithmic
    flops and bytes per launch, achieved rates and their fractions of the class's pipe
    peak and of HBM; 'bound' is the roof nearer to being reached."""
    total = sum(v["ms"] for v in prof.values()) or 1.0
    out = {}
    for name, v in prof.items():
        if v["launches"] == 0 or v["ms"] <= 0:
            continue
        s = v["ms"] * 1e-3
        peak_key, pipe = _PIPE[name]
        tfl = v["flops"] / s / 1e12
        gbs = v["bytes"] / s / 1e9
        e = {"kernel": _KERNEL[name], "launches": v["launches"], "ms": v["ms"], "share_of_profiled": v["ms"] / total,
             "launch_avg_ms": v["ms"] / v["launches"], "flops_per_launch": v["flops"] / v["launches"],
             "bytes_per_launch": v["bytes"] / v["launches"], "achieved_tflops": tfl, "achieved_gbs": gbs,
             "frac_hbm": gbs / peaks["hbm_gbs"]}
        if peak_key:
            e["pipe"] = pipe
            e["pipe_peak_tflops"] = peaks[peak_key]
            e["frac_pipe"] = tfl / peaks[peak_key]
        e["bound"] = pipe if peak_key and e["frac_pipe"] >= e["frac_hbm"] else "hbm"
        if name in _LIMIT:
            e["limited_by"] = _LIMIT[name]
        out[name] = e
    return out


def roofline_entry(rooflines, peaks, traffic=None):
    """The dominant kernel of the step (largest event-timed share) in the bench schema."""
    name, e = max(rooflines.items(), key=lambda kv: kv[1]["ms"])
    if e["bound"] == "hbm":
        achieved, peak, unit, frac = e["achieved_gbs"], peaks["hbm_gbs"], "GB/s", e["frac_hbm"]
    else:
        achieved, peak, unit, frac = e["achieved_tflops"], e["pipe_peak_tflops"], "TFLOP/s", e["frac_pipe"]
    return {"bound": e["bound"], "kernel": e["kernel"], "achieved": achieved, "peak": peak, "unit": unit,
            "frac": frac, "traffic": traffic, "limited_by": e.get("limited_by"), "launch_avg_ms": e["launch_avg_ms"],
            "flops_per_launch": e["flops_per_launch"], "bytes_per_launch": e["bytes_per_launch"],
            "share_of_step": e["share_of_profiled"],
            "timing": "CUDA events on the library stream around each launch / sweep graph inside one mixed B=16 layer",
            "peak_source": peaks["source"]}


def parity_vs_oracle(ctx, n_layers=10):
    """Plain FP64 GPU against the oracle over the workload's first ten layers from the
    initial state: ⟨ψ|ψ⟩ relative error, max |Δ⟨Z_i⟩|, equal bonds, and the smallest
    relative gap (σ_χ − σ_χ+1)/σ_χ over the layer's truncated cuts."""
    import tenetgb
    from oracle import tenet_oracle as O
    from tenetgb import workloads as W

    sites, layers = W.tebd_workload(L=L_SITES, chi0=CHI0, n_layers=n_layers)
    Z = W.pauli_z()
    psi = tenetgb.MPS(sites, ctx=ctx, max_bond=CHI_MAX, precision="native")
    ref = O.OMPS([a.copy() for a in sites])
    rows = []
    t0 = time.perf_counter()
    for ell, ly in enumerate(layers):
        psi.evolve_brickwork_([ly], maxdim=CHI_MAX, threshold=CUTOFF)
        spectra = []
        O.tebd(ref, [ly], CHI_MAX, CUTOFF, spectra=spectra)
        ov, ov_o = psi.overlap(psi), O.overlap(ref, ref)
        z_o, _ = O.local_expectations(ref, Z)
        gaps = [g for g in (O.truncation_gap(x, CHI_MAX, CUTOFF) for x in spectra) if np.isfinite(g)]
        rows.append({"layer": ell + 1, "overlap_rel_err": abs(ov - ov_o) / abs(ov_o),
                     "z_max_abs_err": float(np.abs(psi.local_expectations(Z) - z_o).max()),
                     "bonds_equal": psi.bondsizes() == ref.bondsizes(), "truncated_cuts": len(gaps),
                     "min_relative_gap": min(gaps) if gaps else None})
    return {"layers": rows, "max_overlap_rel_err": max(r["overlap_rel_err"] for r in rows),
            "max_z_abs_err": max(r["z_max_abs_err"] for r in rows),
            "all_bonds_equal": all(r["bonds_equal"] for r in rows), "seconds": time.perf_counter() - t0,
            "oracle": "numpy/LAPACK restatement (zgesdd), all host cores"}


def run_ours(args):
    import torch

    import tenetgb
    from tenetgb import workloads as W

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    dev = torch.device("cuda", local)
    ctx = tenetgb.Context(local)
    ctx.set_autotune(True)  # launch shapes are tuned on first use (saturation / warm-up)
    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    l2buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2

    n_layers = SAT_LAYERS + args.warmup + args.steps + 1
    all_layers = layers_for(n_layers)
    Bt = args.batch
    insts = [W.random_mps_arrays(L_SITES, 2, CHI0, seed=2 + 1000 * b) for b in range(Bt)]
    base = tenetgb.MPS.batched(insts, ctx=ctx, max_bond=CHI_MAX, precision="native")
    base.evolve_brickwork_(all_layers[:SAT_LAYERS], maxdim=CHI_MAX, threshold=CUTOFF)
    ctx.sync()
    host_states = [base.sites(b) for b in range(Bt)]
    host_state = host_states[0]
    run_layers = all_layers[SAT_LAYERS:SAT_LAYERS + args.warmup + args.steps]
    prof_layer = all_layers[-1]

    def timed(psi, layers, warm):
        return _timed_layers(ctx, torch, stream, dev, l2buf, psi, layers, warm)

    # mixed (headline) on a device copy of the saturated state
    psi_mixed = base.copy()
    psi_mixed.set_precision("mixed")
    launches0 = ctx.launches()
    with ClockSampler(local) as clk:
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        t_mixed = timed(psi_mixed, run_layers, args.warmup)
        torch.cuda.synchronize(dev)
    launches_total = ctx.launches() - launches0
    launches_per_step = launches_total / max(1, len(run_layers))
    # the same layers applied left to right (each layer first moves the centre back
    # across the chain): the gate order the layers had before the serpentine sweep
    psi_lr = base.copy()
    psi_lr.set_precision("mixed")
    t_lr = timed(psi_lr, [(ly[0], ly[1], False) for ly in run_layers], args.warmup)
    del psi_lr
    # one more mixed layer with the phase profiler on: each Jacobi sweep graph, GEMM and QR
    # of the step bracketed by CUDA events on the library stream (outside the timed region)
    peaks = pipe_peaks(ctx)
    prof_psi = psi_mixed.copy()
    ctx.profile(True)
    ctx.refine_stats(reset=True)
    prof_psi.evolve_brickwork_([prof_layer], maxdim=CHI_MAX, threshold=CUTOFF)
    prof = ctx.profile_read()
    refine = ctx.refine_stats(reset=True)
    ctx.profile(False)
    del prof_psi
    rooflines = kernel_rooflines(prof, peaks)
    # plain FP64, one instance (instance 0's saturated state), the same layers
    psi_fp64 = tenetgb.MPS(host_state, ctx=ctx, max_bond=CHI_MAX, precision="native")
    t_fp64 = timed(psi_fp64, run_layers, args.warmup)
    # plain FP64 with the B instances batched (1 warm-up layer, 2 timed): the batching
    # share of the mixed-batched speed-up
    psi_fp64b = base.copy()
    t_fp64b = timed(psi_fp64b, run_layers[:3], 1)
    del psi_fp64b
    # accuracy of mixed vs FP64 after the same layers (instance 0)
    m0 = tenetgb.MPS(psi_mixed.sites(0), ctx=ctx, max_bond=CHI_MAX)
    ov_m, ov_f = m0.overlap(m0), psi_fp64.overlap(psi_fp64)
    cross = m0.overlap(psi_fp64)
    z_m = m0.local_expectations(W.pauli_z())
    z_f = psi_fp64.local_expectations(W.pauli_z())
    del m0
    # e2e through the public API from page-locked host buffers: every step uploads all
    # instances' sites, runs the layer, and downloads the new sites (double-buffered pinned
    # copies sized for the largest bonds)
    t_e2e, h2d, d2h = [], 0, 0
    caps = [min(CHI_MAX, 2 ** min(k, L_SITES - k)) for k in range(L_SITES + 1)]

    def pinned_sites():
        return [[torch.empty(2 * caps[i] * 2 * caps[i + 1], dtype=torch.float64, pin_memory=True).numpy()
                 .view(np.complex128) for i in range(L_SITES)] for _ in range(Bt)]

    bufs = [pinned_sites(), pinned_sites()]
    states = []
    for b, st in enumerate(host_states):
        row = []
        for i, a in enumerate(st):
            v = bufs[0][b][i][: a.size].reshape(a.shape, order="F")
            v[...] = a
            row.append(v)
        states.append(row)
    e2e_layers = run_layers[: 1 + min(args.steps, 4)]
    for k, ly in enumerate(e2e_layers):
        dst = bufs[(k + 1) % 2]
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        psi = tenetgb.MPS.batched(states, ctx=ctx, max_bond=CHI_MAX, precision="mixed")
        psi.evolve_brickwork_([ly], maxdim=CHI_MAX, threshold=CUTOFF)
        new_states = [psi.sites(b, out=dst[b]) for b in range(Bt)]
        dt = time.perf_counter() - t0
        del psi
        if k >= 1:
            t_e2e.append(dt)
            h2d = sum(s.nbytes for st in states for s in st) + sum(np.asarray(g).nbytes for g in ly[1])
            d2h = sum(s.nbytes for st in new_states for s in st)
        states = new_states
    # algorithmic work of the timed layers (tenetgb.flops_bytes: two QR moves, θ, the gate
    # and the Golub–Reinsch SVD count per gate) on the saturated bonds
    from tenetgb import flops_bytes as F

    sat_bonds = base.bondsizes()
    timed_layers = run_layers[args.warmup:]
    layer_flops = [F.tebd_layer(sat_bonds, ly[0], len(ly[1])) for ly in timed_layers]
    # max over ranks
    K = args.steps
    tm, tf, tfb, te = max_over_ranks([sum(t_mixed), sum(t_fp64) / len(t_fp64) * K,
                                      sum(t_fp64b) / len(t_fp64b) * K, sum(t_e2e) / len(t_e2e) * K], ws)
    value = replica_throughput(ws, Bt, K, tm)
    fp64_value = replica_throughput(ws, 1, K, tf)
    fp64b_value = replica_throughput(ws, Bt, K, tfb)
    out = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": ws,
        "steps": K,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * tm / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c64 (FP32 Jacobi pre-pass; split-BF16 tensor-core GEMMs; FP64 rotations/truncation/overlaps)",
        "data": "synthetic (seeded Gaussian MPS, Haar gates)",
        "config": bench_config(ws, Bt),
        "algorithmic_tflops": {"mixed_batched": ws * Bt * sum(layer_flops) / tm / 1e12,
                               "fp64": ws * sum(layer_flops) / (sum(t_fp64) / len(t_fp64) * K) / 1e12,
                               "gflop_per_layer_instance": sum(layer_flops) / len(layer_flops) / 1e9,
                               "convention": "two QR gauge moves + theta + gate + Golub-Reinsch SVD per gate, complex "
                                             "MAC = 8 flops (tenetgb.flops_bytes)"},
        "left_to_right": {"value": replica_throughput(ws, Bt, K, sum(t_lr) / len(t_lr) * K), "unit": UNIT,
                          "ms_per_step": 1e3 * sum(t_lr) / len(t_lr),
                          "note": "mixed B=16 with every layer applied left to right"},
        "fp64": {"value": fp64_value, "unit": UNIT, "ms_per_step": 1e3 * tf / K, "instances": 1,
                 "speedup_of_value": value / fp64_value},
        "fp64_batched": {"value": fp64b_value, "unit": UNIT, "ms_per_step": 1e3 * tfb / K, "instances": Bt,
                         "layers_timed": len(t_fp64b),
                         "speedup_batching": fp64b_value / fp64_value, "speedup_precision": value / fp64b_value},
        "accuracy_mixed_vs_fp64": {
            "overlap_rel_err": abs(ov_m - ov_f) / abs(ov_f),
            "fidelity_1_minus": float(1 - abs(cross) ** 2 / (abs(ov_m) * abs(ov_f))),
            "z_max_abs_err": float(np.abs(z_m - z_f).max()),
            "layers_compared": len(run_layers),
        },
        "e2e": {"value": replica_throughput(ws, Bt, K, te), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "layers_timed": len(t_e2e)},
        "gpu_launches": int(round(launches_per_step * K)),
        "clocks": clk.summary(),
        "roofline": roofline_entry(rooflines, peaks, traffic=DOMINANT_TRAFFIC.get(max(rooflines, key=lambda k: rooflines[k]["ms"]))),
        "kernel_rooflines": rooflines,
        "refinement": dict(refine, per_call_iterations=refine["iterations"] / max(1, refine["calls"]),
                           note="truncated mixed SVDs of the profiled layer (one per gate, B instances each)"),
        "peaks": peaks,
    }
    if rank == 0:
        if not args.quick:
            print("bench: parity", file=sys.stderr, flush=True)
            out["parity_fp64_vs_oracle"] = parity_vs_oracle(ctx)
        print("bench: cpu sample", file=sys.stderr, flush=True)
        out["cpu_baseline"] = cpu_sample(host_state, run_layers[0])
        if not args.quick:
            out["configs"] = other_configs(args, ctx, torch, stream, peaks)
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def cpu_sample(host_state, layer):
    """Oracle (numpy/LAPACK restatement, all host cores) on one whole saturated layer
    applied to the same input state."""
    from oracle import tenet_oracle as O

    gates = layer[1]
    psi = O.OMPS([np.ascontiguousarray(s) for s in host_state])
    t0 = time.perf_counter()
    O.tebd(psi, [layer], maxdim=CHI_MAX, threshold=CUTOFF)
    dt = time.perf_counter() - t0
    return {"value": 1.0 / dt, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": f"all {len(gates)} gates of one saturated layer (same input MPS), numpy/LAPACK, "
                      f"{os.cpu_count()} threads"}


def run_reference(args):
    """The reference algorithm's CPU path (the oracle restatement: numpy/LAPACK on all
    host cores) on the same workload: after the five saturating layers, every step
    applies one whole brickwork layer (31-32 gates), as a step of the GPU arm does."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import tenet_oracle as O
    from tenetgb import workloads as W

    all_layers = layers_for(SAT_LAYERS + args.warmup + args.steps)
    psi = O.OMPS(W.random_mps_arrays(L_SITES, 2, CHI0, seed=2))
    O.tebd(psi, all_layers[:SAT_LAYERS], maxdim=CHI_MAX, threshold=CUTOFF)
    from tenetgb import flops_bytes as F

    times, flops = [], 0.0
    for k, ly in enumerate(all_layers[SAT_LAYERS:]):
        fl = F.tebd_layer(psi.bondsizes(), ly[0], len(ly[1]))
        t0 = time.perf_counter()
        O.tebd(psi, [ly], maxdim=CHI_MAX, threshold=CUTOFF)
        if k >= args.warmup:
            times.append(time.perf_counter() - t0)
            flops += fl
    t = sum(times)
    value = args.steps / t
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 (FP64)", "data": "synthetic (seeded Gaussian MPS, Haar gates)", "impl": "reference",
        "config": bench_config(ws, args.batch),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                         "sample": "whole saturated brickwork layers (31-32 gates) per step, one MPS, numpy/LAPACK "
                                   f"on {os.cpu_count()} threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "algorithmic_tflops": flops / t / 1e12,
    }
    print(json.dumps(out), flush=True)


def run_plain_small(args, ctx=None):
    """Config 1 (plain FP64, small): L=32, d=2, χ=64 Gaussian MPS (seed 1, not
    orthogonalised): the QR left-canonize sweep canonize!(ψ, site 32), overlap(ψ, ψ) and
    ⟨ψ|Z₁₆|ψ⟩ = overlap(ψ, Z₁₆ψ) with Z₁₆ψ from the one-site simple_update!.  Latency-bound:
    median µs per operation over 20 repetitions and kernel launches per operation, with
    the values checked against the oracle."""
    import tenetgb
    from oracle import tenet_oracle as O
    from tenetgb import workloads as W

    if ctx is None:
        ctx = tenetgb.Context(0)
    sites = W.plain_small_workload()
    Z = W.pauli_z()

    def op_canonize():
        p = tenetgb.MPS(sites, ctx=ctx)
        ctx.sync()
        l0, t0 = ctx.launches(), time.perf_counter()
        p.canonize_(32)
        ctx.sync()
        return time.perf_counter() - t0, ctx.launches() - l0, p

    res, psi = {}, None
    for name in ("canonize", "overlap", "z16"):
        ts, ls = [], []
        for _ in range(21):
            if name == "canonize":
                dt, nl, psi = op_canonize()
            elif name == "overlap":
                l0, t0 = ctx.launches(), time.perf_counter()
                ov = psi.overlap(psi)
                dt, nl = time.perf_counter() - t0, ctx.launches() - l0
            else:
                l0, t0 = ctx.launches(), time.perf_counter()
                zp = psi.copy()
                zp.simple_update_(Z, [16])
                z = psi.overlap(zp)
                dt, nl = time.perf_counter() - t0, ctx.launches() - l0
            ts.append(dt)
            ls.append(nl)
        res[name] = {"us": 1e6 * float(np.median(ts[1:])), "launches": int(np.median(ls[1:]))}
    ref = O.OMPS([a.copy() for a in sites])
    O.canonize(ref, 32)
    ov_o = O.overlap(ref, ref)
    pz = ref.copy()
    O.simple_update(pz, Z, [16])
    z_o = O.overlap(ref, pz)
    return {"metric": "plain_small_latency_us", "config": {"workload": "plain_L32_d2_chi64_seed1", "L": 32, "chi": 64},
            "ops": res, "overlap_rel_err_vs_oracle": abs(ov - ov_o) / abs(ov_o),
            "z16_rel_err_vs_oracle": abs(z - z_o) / abs(ov_o), "dtype": "c128 (FP64)",
            "note": "latency-bound (tiny): µs and launches per operation, no roofline claim"}


def other_configs(args, ctx, torch, stream, peaks):
    """Configs 1, 3, 4 and 5 and the standalone kernel rooflines, each compact, for the
    one bench line (each is also a --workload of its own)."""
    out = {}
    for name, fn in [("plain_small", lambda: run_plain_small(args, ctx)),
                     ("lattice_8x8", lambda: run_lattice(args, ctx, stream)),
                     ("kernels", lambda: run_kernels(args, ctx, stream)),
                     ("batched_512", lambda: run_batched(args, ctx)),
                     ("serving", lambda: run_serving(args, rates=(1000, 5000)))]:
        print(f"bench: {name}", file=sys.stderr, flush=True)
        t0 = time.perf_counter()
        try:
            r = fn()
        except Exception as e:  # a failing secondary config is reported, not fatal to the headline
            r = {"error": f"{type(e).__name__}: {e}"}
        r["seconds"] = time.perf_counter() - t0
        if name == "batched_512":
            for k in ("config",):
                r[k] = {kk: vv for kk, vv in r.get(k, {}).items() if kk not in ("Ls", "chis")}
        if name == "serving":
            r.pop("config", None)
        out[name] = r
    return out


def profile_gate(args):
    """One saturated two-site gate (θ 512×512) on a χ=256 random MPS of 20 sites: the
    small case for ncu captures.  Runs the gate twice (the first builds the cached CUDA
    graphs and runs the autotuner) and prints the second gate's time; the second gate is
    bracketed by cudaProfilerStart/Stop."""
    import torch

    import tenetgb
    from tenetgb import workloads as W

    ctx = tenetgb.Context(0)
    ctx.set_autotune(True)
    insts = [W.random_mps_arrays(20, 2, CHI_MAX, seed=7 + b) for b in range(args.batch)]
    gate = W.gate_tensor(W.haar_unitary(np.random.default_rng(8), 4))
    psi = tenetgb.MPS.batched(insts, ctx=ctx, max_bond=CHI_MAX, precision=args.precision)
    psi.canonize_([10, 11])
    for rep in range(2):
        ctx.sync()
        if rep == 1:  # `ncu --profile-from-start off` captures only this gate
            torch.cuda.profiler.start()
        t0 = time.perf_counter()
        psi.simple_update_(gate, [10, 11], maxdim=CHI_MAX, threshold=CUTOFF)
        ctx.sync()
        dt = time.perf_counter() - t0
        if rep == 1:
            torch.cuda.profiler.stop()
    print(json.dumps({"profile_gate_ms": 1e3 * dt, "precision": args.precision, "batch": args.batch,
                      "bond": psi.bondsizes()[9], "launches": ctx.launches()}))


def profile_layer(args):
    """One brickwork layer (odd bonds, 10 gates) on B saturated random MPS of 20 sites,
    χ = 256 (θ 512×512 per gate): the small case for the launch list of the headline step.
    The first layer builds the cached graphs; the second is bracketed by
    cudaProfilerStart/Stop."""
    import torch

    import tenetgb
    from tenetgb import workloads as W

    ctx = tenetgb.Context(0)
    insts = [W.random_mps_arrays(20, 2, CHI_MAX, seed=7 + b) for b in range(args.batch)]
    layers = W.tebd_layers(20, 3)
    psi = tenetgb.MPS.batched(insts, ctx=ctx, max_bond=CHI_MAX, precision=args.precision)
    for rep, ly in enumerate([layers[0], layers[2]]):
        ctx.sync()
        if rep == 1:
            torch.cuda.profiler.start()
        t0 = time.perf_counter()
        psi.evolve_brickwork_([ly], maxdim=CHI_MAX, threshold=CUTOFF)
        ctx.sync()
        dt = time.perf_counter() - t0
        if rep == 1:
            torch.cuda.profiler.stop()
    print(json.dumps({"profile_layer_ms": 1e3 * dt, "precision": args.precision, "batch": args.batch,
                      "gates": len(layers[2][1]), "launches": ctx.launches()}))


def profile_svd(args):
    """The roofline kernel's own workload: tensor_svd_thin of one 512×512 C64 Gaussian
    matrix in FP64 (U, S and V), run twice; the second call is bracketed by
    cudaProfilerStart/Stop (small ncu case for the k_jacobi_step_reg traffic)."""
    import torch

    import tenetgb

    ctx = tenetgb.Context(0)
    rng = np.random.default_rng(0)
    A = tenetgb.DeviceTensor.from_numpy(ctx, rng.standard_normal((512, 512)) + 1j * rng.standard_normal((512, 512)),
                                        ["r", "c"])
    for rep in range(2):
        ctx.sync()
        if rep == 1:
            torch.cuda.profiler.start()
        t0 = time.perf_counter()
        tenetgb.tensor_svd_thin(A, ["r"], ["c"], "s")
        ctx.sync()
        dt = time.perf_counter() - t0
        if rep == 1:
            torch.cuda.profiler.stop()
    print(json.dumps({"profile_svd_ms": 1e3 * dt, "m": 512, "n": 512}))


def profile_dmrg(args):
    """One saturated dmrg!(ψ, H, 1; Dmrg2, maxdim = 128) call on the 100-site Ising chain:
    five untimed calls from the product state saturate the bonds, the sixth is bracketed by
    cudaProfilerStart/Stop (launch list of one sweep)."""
    import torch

    import tenetgb

    n, chi = 100, 128
    ctx = tenetgb.Context(0)
    H = tenetgb.ising_1d_mpo(n, 1.0, 1.0)
    psi = tenetgb.MPS([np.array([1.0, 0.0], dtype=np.complex128).reshape(1, 2, 1) for _ in range(n)], ctx=ctx)
    for rep in range(6):
        ctx.sync()
        if rep == 5:
            l0 = ctx.launches()
            torch.cuda.profiler.start()
        t0 = time.perf_counter()
        _, E = tenetgb.dmrg_(psi, H, 1, method=tenetgb.Dmrg2, maxdim=chi)
        ctx.sync()
        dt = time.perf_counter() - t0
        if rep == 5:
            torch.cuda.profiler.stop()
    print(json.dumps({"profile_dmrg_ms": 1e3 * dt, "energy": float(E), "launches": ctx.launches() - l0,
                      "bond_max": max(psi.bondsizes())}))


def run_lattice(args, ctx=None, stream=None):
    """Closed 8×8 lattice, bond 8, ComplexF32 (seed 4): contraction to a scalar along the
    planner's path, in 3×TF32 (tensor pipe), TF32, FP32 (CUDA cores) and FP64; errors
    against the FP64 run.  Returns one JSON-able dict (a secondary workload)."""
    import torch

    import tenetgb
    from tenetgb import network as N

    if ctx is None:
        ctx = tenetgb.Context(0)
        stream = torch.cuda.Stream()
        ctx.set_stream(stream.cuda_stream)
    net = N.lattice_2d(8, 8, 8, seed=4)
    path = N.greedy_path(net.labels, net.dims)
    steps, peak = N.path_flops(net.labels, net.dims, path)
    flops = sum(st["flops"] for st in steps)
    res = {}
    for mode, dt in [("fp64", np.complex128), ("3xtf32", np.complex64), ("tf32", np.complex64), ("fp32", np.complex64)]:
        prec = {"fp64": "native", "3xtf32": "mixed", "tf32": "tf32", "fp32": "native"}[mode]
        N.contract(net, path, precision=prec, dtype=dt, ctx=ctx)  # warm-up
        ctx.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        val = N.contract(net, path, precision=prec, dtype=dt, ctx=ctx)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        res[mode] = {"ms": ms, "value": complex(val), "tflops": flops / (ms * 1e-3) / 1e12}
    ref = res["fp64"]["value"]
    for mode in res:
        res[mode]["rel_err_vs_fp64"] = abs(res[mode]["value"] - ref) / abs(ref)
        res[mode]["value"] = [res[mode]["value"].real, res[mode]["value"].imag]
    return {"metric": "lattice_8x8_bond8_contraction_tflops", "value": res["3xtf32"]["tflops"],
            "unit": "TFLOP/s (complex-algorithmic)", "steps": len(path), "peak_elements": peak,
            "path_flops": flops, "modes": res, "data": "synthetic (seeded Gaussian C32, seed 4)"}


def run_kernels(args, ctx=None, stream=None):
    """Kernel rooflines outside the TEBD step: the permutation kernel on 1 GiB ComplexF64
    tensors (bytes = 2·numel·16, against the measured HBM copy rate) and the contraction
    GEMMs at 4096³ (C32 on the tcgen05 tensor pipe in TF32 and 3×TF32, counted as real
    tensor-core flops 2·(2m)·n·(2k) per pass against half the measured BF16 rate, the
    dense TF32 rate; C64 on the FP64 pipe).  Each figure is the best of 5 launches timed
    with CUDA events.  Prints one JSON line (a secondary workload)."""
    import ctypes as C

    import torch

    import tenetgb

    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}
    hbm, tf32 = peaks["hbm_gbs"], peaks["bf16_tflops"] / 2
    if ctx is None:
        ctx = tenetgb.Context(0)
        stream = torch.cuda.Stream()
        ctx.set_stream(stream.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def best(fn, reps=5):
        fn()
        ctx.sync()
        ts = []
        for _ in range(reps):
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return min(ts)

    out = {"permute": [], "gemm": []}
    for dims, perm in [((1024, 1024, 64), (2, 0, 1)), ((1024, 1024, 64), (1, 0, 2)), ((64, 2, 1024, 2, 256), (2, 0, 4, 1, 3)),
                       ((512, 512, 256), (0, 2, 1))]:
        numel = int(np.prod(dims))
        src = ctx.alloc(numel * 16)
        dst = ctx.alloc(numel * 16)
        rank = len(dims)
        cd = (C.c_int64 * rank)(*dims)
        st = [1]
        for x in dims[:-1]:
            st.append(st[-1] * x)
        cs = (C.c_int64 * rank)(*st)
        cp = (C.c_int32 * rank)(*perm)

        def f():
            ctx.check(ctx.lib.tn_permute(ctx.h, 3, rank, cd, cs, cp, C.c_void_p(src), C.c_void_p(dst), 0))

        ms = best(f)
        gbs = 2 * numel * 16 / (ms * 1e-3) / 1e9
        out["permute"].append({"dims": list(dims), "perm": list(perm), "ms": ms, "GB/s": gbs, "frac_hbm": gbs / hbm})
        ctx.free(src)
        ctx.free(dst)
    N = 4096
    one, zero = (C.c_double * 2)(1, 0), (C.c_double * 2)(0, 0)
    for dt, prec, label, passes in [(2, 2, "c32_tf32", 1), (2, 1, "c32_3xtf32", 3), (2, 0, "c32_fp32_cuda_cores", 0),
                                    (3, 0, "c64_fp64", 0)]:
        n = N if dt == 2 else 2048
        tdt = torch.complex64 if dt == 2 else torch.complex128
        A = torch.randn(n, n, dtype=tdt, device="cuda")
        B = torch.randn(n, n, dtype=tdt, device="cuda")
        Cc = torch.empty(n, n, dtype=tdt, device="cuda")
        torch.cuda.synchronize()

        def g():
            ctx.check(ctx.lib.tn_gemm(ctx.h, dt, prec, b"N", b"N", n, n, n, one, C.c_void_p(A.data_ptr()), n, 0,
                                      C.c_void_p(B.data_ptr()), n, 0, zero, C.c_void_p(Cc.data_ptr()), n, 0, 1))

        ms = best(g)
        cplx = 8 * n**3 / (ms * 1e-3) / 1e12
        e = {"kind": label, "n": n, "ms": ms, "complex_algorithmic_tflops": cplx}
        if passes:
            real = passes * 2 * (2 * n) * n * (2 * n) / (ms * 1e-3) / 1e12
            e.update({"tensor_tflops": real, "frac_tf32_peak": real / tf32})
        out["gemm"].append(e)
        del A, B, Cc
    return {"metric": "kernel_rooflines", "hbm_peak_gbs": hbm, "tf32_dense_peak_tflops": tf32,
            "bf16_dense_peak_tflops": peaks["bf16_tflops"],
            "peak_source": "MEASURED_PEAKS.json (TF32 dense = BF16 / 2)", **out}


def batched_flops(Ls, chis, maxdims, d=2):
    """Algorithmic flops of canonize!(ψ, L) → compress!(ψ; maxdim) for the given shapes
    (tenetgb.flops_bytes conventions)."""
    from tenetgb import flops_bytes as F
    from tenetgb import workloads as W

    return sum(F.canonize_compress(L, W.clamped_bonds(L, d, chi), md, d) for L, chi, md in zip(Ls, chis, maxdims))


def run_batched(args, ctx=None):
    """Config 4: ragged batch of random MPS (L uniform in [16, 128], χ log-uniform in
    [16, 512], d=2, seed 5; the first --batched-sample of the 512-MPS population), each
    canonize!(ψ, MixedCanonical(L)) → compress!(ψ; maxdim = χ÷2) → norm(ψ), FP64.  The
    grouped path (one launch per kernel per sweep step over all instances) against the
    per-instance device loop on the first --batched-loop instances of the sample.
    Returns one JSON-able dict (a secondary workload)."""
    import torch

    import tenetgb
    from tenetgb import workloads as W
    from tenetgb.group import MPSGroup

    Ls_all, chis_all = W.batched_population()
    n = args.batched_sample
    Ls, chis = Ls_all[:n], chis_all[:n]
    maxdim = [max(1, c // 2) for c in chis]
    if ctx is None:
        ctx = tenetgb.Context(0)
        ctx.set_autotune(True)
    g = MPSGroup.random(Ls, chis, seed=5, ctx=ctx)
    ctx.sync()
    init = [g.sites(b) for b in range(n)]
    flops = batched_flops(Ls, chis, maxdim)
    sampler = ClockSampler(0)
    times_g, times_p = [], []
    with sampler:
        # warm-up on the first 64 instances (graphs, launch tuning), then the whole sample
        wn = min(n, 64)
        gw = MPSGroup.random(Ls[:wn], chis[:wn], seed=5, ctx=ctx)
        gw.canonize_compress_norm(maxdim[:wn])
        del gw
        ctx.check(ctx.lib.tn_group_fill_random(g.h, 5))
        ctx.sync()
        t0 = time.perf_counter()
        norms_g = g.canonize_compress_norm(maxdim)
        times_g.append(time.perf_counter() - t0)
        nl = min(n, args.batched_loop)
        for rep in range(2 if nl <= 8 else 1):
            psis = [tenetgb.MPS([a.copy() for a in init[b]], ctx=ctx) for b in range(nl)]
            ctx.sync()
            t0 = time.perf_counter()
            norms_p = []
            for b, psi in enumerate(psis):
                psi.canonize_(tenetgb.MixedCanonical(Ls[b]))
                psi.compress_(maxdim=maxdim[b])
                norms_p.append(psi.norm())
            times_p.append(time.perf_counter() - t0)
            del psis
    tg, tp = times_g[-1], times_p[-1]
    norms_p = np.array(norms_p)
    # the grouped path restricted to the loop's instances, for a like-for-like speed-up
    fl_loop = batched_flops(Ls[:nl], chis[:nl], maxdim[:nl])
    # CPU oracle on the smallest instances of the sample, ~20 s
    from oracle import tenet_oracle as O

    order = np.argsort([L * c**3 for L, c in zip(Ls, chis)])
    done, spent, fl_cpu = 0, 0.0, 0.0
    for b in order:
        psi = O.OMPS([a.copy() for a in init[b]])
        t0 = time.perf_counter()
        O.canonize(psi, O.MixedCanonical(Ls[b]))
        O.compress(psi, maxdim=maxdim[b])
        O.norm(psi)
        spent += time.perf_counter() - t0
        done += 1
        fl_cpu += batched_flops([Ls[b]], [chis[b]], [maxdim[b]])
        if spent > args.batched_cpu_s:
            break
    return {
        "metric": "batched_canonize_compress_norm_mps_per_s", "value": n / tg, "unit": "MPS/s",
        "higher_is_better": True, "dtype": "c128 (FP64)",
        "data": "synthetic (seeded Gaussian MPS generated on the device, seed 5)",
        "config": {"workload": "ragged_mps_L16to128_chi16to512_canonize_compress_half_norm",
                   "population": 512, "sample": n, "Ls": Ls, "chis": chis, "maxdim": "chi // 2"},
        "grouped": {"s": tg, "mps_per_s": n / tg, "tflops_algorithmic": flops / tg / 1e12},
        "per_instance_loop": {"instances": nl, "s": tp, "mps_per_s": nl / tp,
                              "tflops_algorithmic": fl_loop / tp / 1e12},
        "speedup_grouped_vs_loop_per_flop": (flops / tg) / (fl_loop / tp),
        "norm_max_rel_diff_grouped_vs_loop": float(np.max(np.abs(norms_g[:nl] - norms_p) / norms_p)),
        "algorithmic_flops": flops, "clocks": sampler.summary(),
        "cpu_baseline": {"value": fl_cpu / spent / 1e12, "unit": "TFLOP/s (algorithmic)", "cores": os.cpu_count(),
                         "kind": "port", "sample": f"{done} smallest MPS of the sample through the oracle, "
                                                   f"{spent:.1f} s"},
    }


SERVING_RATES = (100, 300, 1000, 3000, 5000)


def _serving_oracle_sample(srv, ids, spec, trace, budget_s=20.0):
    """The reference's per-query algorithms (oracle, numpy on the host cores) on the
    first queries of a trace until ``budget_s`` of compute: amplitude =
    overlap(ProductState, ψ); ⟨O_i⟩ = overlap(ψ, O_i ψ)/overlap(ψ, ψ); overlap(ψ_a, ψ_b).
    Site data comes from the server's pool (download time not counted)."""
    from oracle import tenet_oracle as O

    cache = {}

    def mps(m):
        if m not in cache:
            cache[m] = O.OMPS(srv.sites(ids[m]))
        return cache[m]

    done, spent = 0, 0.0
    for _, kind, m, arg in trace:
        psis = [mps(m)] + ([mps(arg)] if kind == "ovl" else [])
        t0 = time.perf_counter()
        if kind == "amp":
            O.amplitude([np.eye(2, dtype=np.complex128)[b] for b in arg], psis[0])
        elif kind == "exp":
            O.expectation(psis[0], arg[0], arg[1])
        else:
            O.overlap(psis[0], psis[1])
        spent += time.perf_counter() - t0
        done += 1
        if spent >= budget_s:
            break
    return done, spent


def run_serving(args, rates=None):
    """Query serving on a device-resident pool: 16 random MPS (L in [8, 256], χ in
    {32, …, 1024}, d=2, seed 6), Poisson arrivals at each rate of SERVING_RATES (seed
    7+rate), 60 % amplitudes / 30 % ⟨O_i⟩ / 10 % overlaps, FP64.  For each rate: queries/s
    (completed ÷ first submit → last result) and p50 / p99 latency (submit → result on
    the host).  Prints one JSON line (a secondary workload)."""
    import torch

    from tenetgb import serve
    from tenetgb import workloads as W

    spec = W.serving_pool()
    srv = serve.Server(hbm_budget=int(args.serve_budget_gb * 1e9), work_bytes=16 << 30, max_batch=64,
                       precision=args.serve_precision)
    t0 = time.perf_counter()
    ids = [srv.add_random_mps(L, chi, seed=s) for (L, chi, s) in spec]
    reg_s = time.perf_counter() - t0
    pool_L = [L for L, _, _ in spec]
    pool_bytes = srv.stats()["pool_bytes"]
    # warm-up: every pool MPS once per kind
    warm = []
    for m, L in enumerate(pool_L):
        warm.append(srv.submit_amplitude(ids[m], bits=np.zeros(L, np.int64)))
        warm.append(srv.submit_expectation(ids[m], 1, np.eye(2)))
    for p in range(len(ids) // 2):
        warm.append(srv.submit_overlap(ids[2 * p], ids[2 * p + 1]))
    for t in warm:
        srv.wait(t)
    per_rate = []
    sampler = ClockSampler(torch.cuda.current_device() if torch.cuda.is_available() else 0)
    with sampler:
        for rate in (rates or SERVING_RATES):
            trace = W.serving_trace(pool_L, rate, args.queries, seed=7 + rate)
            tickets, t_sub = [], []
            start = time.perf_counter()
            for (ta, kind, m, arg) in trace:
                while time.perf_counter() - start < ta:
                    pass
                t_sub.append(time.perf_counter())
                if kind == "amp":
                    tickets.append(srv.submit_amplitude(ids[m], bits=arg))
                elif kind == "exp":
                    tickets.append(srv.submit_expectation(ids[m], arg[0], arg[1]))
                else:
                    tickets.append(srv.submit_overlap(ids[m], ids[arg]))
            lat = np.array([srv.wait(t)[1] for t in tickets])
            t_done = np.array(t_sub) + lat
            span = float(t_done.max() - min(t_sub))
            kinds = np.array([q[1] for q in trace])
            entry = {"rate": rate, "queries": len(trace), "qps": len(trace) / span,
                     "p50_ms": 1e3 * float(np.percentile(lat, 50)), "p99_ms": 1e3 * float(np.percentile(lat, 99))}
            for k in ("amp", "exp", "ovl"):
                if (kinds == k).any():
                    entry[f"p50_{k}_ms"] = 1e3 * float(np.percentile(lat[kinds == k], 50))
            per_rate.append(entry)
            print(json.dumps(entry), file=sys.stderr, flush=True)
    st = srv.stats()
    cpu_trace = W.serving_trace(pool_L, SERVING_RATES[0], args.queries, seed=7 + SERVING_RATES[0])
    done, spent = _serving_oracle_sample(srv, ids, spec, cpu_trace)
    srv.close()
    best = max(per_rate, key=lambda e: e["qps"])
    return {
        "metric": "serving_queries_per_s", "value": best["qps"], "unit": "queries/s", "higher_is_better": True,
        "dtype": "c128 (FP64)" if args.serve_precision == "native" else
                 "c128 data; FP32 amplitude/overlap sweeps, FP64 <O_i> and results",
        "data": "synthetic (seeded Gaussian MPS generated on the device, seed 6)",
        "config": {"workload": "serving_pool16_L8to256_chi32to1024_mix60amp30exp10ovl", "pool": spec,
                   "pool_bytes": pool_bytes, "registration_s": reg_s, "queries_per_rate": args.queries,
                   "max_batch": 64, "work_bytes": 16 << 30},
        "per_rate": per_rate, "p50_ms_at_best": best["p50_ms"], "p99_ms_at_best": best["p99_ms"],
        "server_stats": st, "clocks": sampler.summary(),
        "cpu_baseline": {"value": done / spent, "unit": "queries/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": f"first {done} queries of the rate-100 trace, the reference's per-query "
                                   f"algorithms in numpy/LAPACK, {spent:.1f} s"},
    }


def run_dmrg(args):
    """2-site DMRG of the 100-site Ising chain (h = J = 1) at χ = 128, the workload of the
    reference's examples/dmrg.ipynb: ``dmrg!(ψ, H, 1; method = Dmrg2(), maxdim = 128)``
    called once per step, starting from the product state |0…0⟩.  Ten calls in all (the
    notebook's count; bonds saturate at 128 after four), the last ``steps`` of them timed
    with CUDA events on the library's stream, L2 flushed between steps.  The energy after
    the tenth call is compared with the notebook's value, -126.96187478469312.  One JSON
    line (a secondary workload)."""
    import torch

    import tenetgb
    from oracle import tenet_oracle as O

    n, chi, total = 100, 128, max(10, args.steps + args.warmup + 4)
    ctx = tenetgb.Context(0)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    H = tenetgb.ising_1d_mpo(n, 1.0, 1.0)
    prod = [np.array([1.0, 0.0], dtype=np.complex128).reshape(1, 2, 1) for _ in range(n)]
    psi = tenetgb.MPS([s.copy() for s in prod], ctx=ctx)
    times, energies = [], []
    launches0 = None
    with ClockSampler(0) as clk:
        for call in range(1, total + 1):
            timed = call > total - args.steps
            with torch.cuda.stream(stream):
                flush_l2(torch, flush)
            ctx.sync()
            if timed and launches0 is None:
                launches0 = ctx.launches()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _, E = tenetgb.dmrg_(psi, H, 1, method=tenetgb.Dmrg2, maxdim=chi)
            e1.record(stream)
            e1.synchronize()
            energies.append(float(E))
            if timed:
                times.append(e0.elapsed_time(e1))
    launches = ctx.launches() - launches0
    ms = float(np.mean(times))
    stats = tenetgb.dmrg_last_stats(ctx)
    # dominant kernel: the pair SVD (k_jacobi_coop, one launch per 256×256 split).
    # Algorithmic flops per launch = sweeps × 255 rounds × 128 pairs × (8m + 24m), m = 256
    # (no right vectors), the sweeps averaged over the call's splits; time per launch =
    # the splits' device time (CUDA events) ÷ the local updates
    sweeps_per_split = stats["svd_sweeps"] / max(1, stats["updates"])
    flops = sweeps_per_split * 255 * 128 * 32 * 256
    split_ms = stats["split_ms"] / max(1, stats["updates"])
    peak = ctx.pipe_peak("fp64")
    achieved = flops / (split_ms * 1e-3) / 1e12
    roofline = {"bound": "fp64_cuda_cores", "kernel": "k_jacobi_coop<double> (FP64 pipe; latency-bound rounds)",
                "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                "peak_source": "FP64 FMA rate of the CUDA cores measured in this run (tn_pipe_peak)",
                "flops_per_launch": flops, "sweeps_per_split": sweeps_per_split, "launch_avg_ms": split_ms,
                "phases_ms_per_step": {k: stats[k] for k in ("canonize_ms", "environments_ms", "eigsolve_ms",
                                                             "split_ms")}}
    # 16 Hamiltonians (h ∈ [0.5, 1.5]) on a batched MPS in lockstep: five untimed calls
    # from the product state, then one timed call
    scan = None
    if args.dmrg_batch > 1:
        fields = np.linspace(0.5, 1.5, args.dmrg_batch)
        q = tenetgb.MPS.batched([[s.copy() for s in prod] for _ in fields], ctx=ctx)
        Hs = [tenetgb.ising_1d_mpo(n, h, 1.0) for h in fields]
        for _ in range(5):
            tenetgb.dmrg_(q, Hs, 1, method=tenetgb.Dmrg2, maxdim=chi)
        with torch.cuda.stream(stream):
            flush_l2(torch, flush)
        ctx.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, Es = tenetgb.dmrg_(q, Hs, 1, method=tenetgb.Dmrg2, maxdim=chi)
        e1.record(stream)
        e1.synchronize()
        sms = e0.elapsed_time(e1)
        scan = {"instances": int(args.dmrg_batch), "fields": [float(fields[0]), float(fields[-1])],
                "value": args.dmrg_batch * 1e3 / sms, "unit": "instance-sweeps/s", "ms_per_step": sms,
                "per_instance_vs_single": (args.dmrg_batch * 1e3 / sms) / (1e3 / ms),
                "energies_per_site": [float(e) / n for e in Es]}
        del q
    # end to end: the MPS from pinned host buffers, one call, the MPS and energy back
    host_sites = [psi.site(i) for i in range(1, n + 1)]
    pinned = [torch.from_numpy(np.asfortranarray(s).reshape(-1, order="F").view(np.float64)).pin_memory()
              for s in host_sites]
    out_bufs = [torch.empty(2 * s.size, dtype=torch.float64, pin_memory=True).numpy().view(np.complex128)
                for s in host_sites]
    h2d = sum(t.numel() * 8 for t in pinned)
    e2e_times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        arrays = [t.numpy().view(np.complex128).reshape(s.shape, order="F") for t, s in zip(pinned, host_sites)]
        q = tenetgb.MPS(arrays, ctx=ctx)
        q.unsafe_setform_(tenetgb.MixedCanonical(1))
        _, Eq = tenetgb.dmrg_(q, H, 1, method=tenetgb.Dmrg2, maxdim=chi)
        back = q.sites(out=out_bufs)
        e2e_times.append(time.perf_counter() - t0)
        del q
    d2h = sum(b.nbytes for b in back) + 8
    # CPU: the oracle on the same saturated state: environments plus the first 40 of the
    # 2(n-1) local updates of one call, extrapolated to the whole call
    tm = {}
    O.dmrg(O.OMPS([s.copy() for s in host_sites], form=O.MixedCanonical(1)), O.ising_1d_mpo(n, 1.0, 1.0), 1,
           method="dmrg2", maxdim=chi, limit=40, timing=tm)
    cpu_s = tm["env_s"] + tm["updates_s"] / max(1, tm["updates"]) * 2 * (n - 1)
    known = -126.96187478469312
    try:  # the notebook's printed energy of every call (tests/golden, extracted from the reference)
        with open(os.path.join(ROOT, "tests", "golden", "reference_known_answers.json")) as f:
            per_call = json.load(f)["dmrg_notebook"]["dmrg2_product"]["energies_per_call"]
    except (OSError, KeyError, ValueError):
        per_call = None
    return {
        "metric": "dmrg2_sweeps_per_s_ising_n100_chi128", "value": 1e3 / ms, "unit": "sweeps/s", "n_gpus": 1,
        "steps": args.steps, "warmup": total - args.steps, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "replicas", "vs_baseline": None, "dtype": "c128 (FP64 GEMMs, Lanczos and Jacobi SVD)",
        "data": "synthetic (Ising MPO h = J = 1, product start state; examples/dmrg.ipynb)",
        "config": {"workload": "dmrg2_ising_n100_chi128", "n": n, "maxdim": chi, "krylovdim": 3, "maxiter": 2,
                   "calls": total, "step": "dmrg!(ψ, H, 1) on the saturated MPS (environments + one sweep)",
                   "l2": "flushed between steps (256 MB write)"},
        "energy_after_10_calls": energies[9], "energy_known_notebook": known,
        "energy_abs_diff": abs(energies[9] - known), "energies": energies,
        "energy_abs_diff_per_call_vs_notebook": ([abs(a - b) for a, b in zip(energies, per_call)]
                                                 if per_call else None),
        "e2e": {"value": 1.0 / float(np.mean(e2e_times)), "unit": "sweeps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches / max(1, args.steps)), "clocks": clk.summary(), "roofline": roofline,
        "batched_scan": scan,
        "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "sweeps/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": "oracle (numpy/LAPACK) on the same saturated MPS: environments + 40 of the 198 "
                                   "local updates of one dmrg!(ψ, H, 1) call, scaled to the call"},
    }


def main():
    # a fatal signal in native code prints the Python stacks of every thread
    faulthandler.enable(file=sys.stderr, all_threads=True)
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="tebd", choices=["tebd", "lattice", "serving", "kernels", "batched", "dmrg", "plain"])
    ap.add_argument("--batched-sample", type=int, default=512, help="instances of the 512-MPS population (batched)")
    ap.add_argument("--batched-loop", type=int, default=16, help="instances of the per-instance device loop (batched)")
    ap.add_argument("--batched-cpu-s", type=float, default=10.0, help="oracle seconds on the smallest instances")
    ap.add_argument("--quick", action="store_true", help="TEBD line only (no parity / secondary configs)")
    ap.add_argument("--queries", type=int, default=200, help="queries per arrival rate (serving)")
    ap.add_argument("--serve-budget-gb", type=float, default=200.0, help="HBM budget of the server (serving)")
    ap.add_argument("--serve-precision", default="native", choices=["native", "mixed"], help="serving arithmetic")
    ap.add_argument("--profile-gate", action="store_true", help="one saturated gate (small ncu case)")
    ap.add_argument("--profile-svd", action="store_true", help="the roofline kernel's SVD (small ncu case)")
    ap.add_argument("--profile-layer", action="store_true", help="one brickwork layer, 20 sites (launch list)")
    ap.add_argument("--profile-dmrg", action="store_true", help="one saturated 2-site DMRG sweep (launch list)")
    ap.add_argument("--precision", default="native", choices=["native", "mixed"])
    ap.add_argument("--batch", type=int, default=16, help="MPS instances advanced in lockstep")
    ap.add_argument("--dmrg-batch", type=int, default=16, help="Hamiltonians of the batched DMRG scan (dmrg)")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.profile_gate:
        profile_gate(args)
    elif args.profile_svd:
        profile_svd(args)
    elif args.profile_layer:
        profile_layer(args)
    elif args.profile_dmrg:
        profile_dmrg(args)
    elif args.workload == "lattice":
        print(json.dumps(run_lattice(args)))
    elif args.workload == "serving":
        print(json.dumps(run_serving(args)))
    elif args.workload == "kernels":
        print(json.dumps(run_kernels(args)))
    elif args.workload == "batched":
        print(json.dumps(run_batched(args)))
    elif args.workload == "dmrg":
        print(json.dumps(run_dmrg(args)))
    elif args.workload == "plain":
        print(json.dumps(run_plain_small(args)))
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
