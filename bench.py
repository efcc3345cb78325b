"""Throughput benchmark of the pulse-signal likelihood hot path.

Workload (the batched configuration): V parameter vectors drawn from the
prior (M U(1,3) Msun, R U(3 r_g, 16 km), spin U(200,600) Hz, cos i U(0,1),
D 1 kpc; two Num4D hot regions, one circular and one with an omitted
crescent; colatitudes U(0,pi), radii U(0.01,0.5), log T U(5.8,6.6)), model
resolution sqrt_num_cells 64 (max 128), num_leaves 128, num_rays 1024,
128 energies; 35x14x67x166 FP64 atmosphere table; 1500 x 128 response;
32 phase bins; counts drawn from the model of the full-size configuration's
vector.  A step is one pass of the hot path -- rays, integrator, energy
integration, response fold, background-marginalised likelihood -- over the
batch.  Meshes are built on the host before the timed region (both arms).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--vectors V]
                    [--impl gb300|reference]

Prints one JSON line (rank 0).  --impl reference times the CPU restatement
of the reference path (oracle/) on the host cores.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "likelihood evals/s at |ΔlogL|≤1e-3 vs FP64, batched vs plain GPU; p50/p99 latency"
UNIT = "likelihood evals/s"
WORKLOAD = ("batched prior vectors of the full-size plain model (2 Num4D hot regions, one "
            "omitted crescent; 64/128 cells, 128 leaves, 1024 rays, 128 energies, 1500x128 "
            "response, 32 bins)")


def peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, gpu_index=0):
        self.cmd = ["nvidia-smi", "-i", str(gpu_index),
                    "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
                    "clocks_event_reasons.hw_thermal_slowdown,"
                    "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                    "--format=csv,noheader,nounits", "-lms", "200"]
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(self.cmd, stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
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
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[2:]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def build_workload(V, seed_vectors=3):
    from xpsi_gb300 import synthetic as SY
    model = SY.config2_model()
    params = SY.config3_vectors(V, seed=seed_vectors)
    return model, params


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("XPSI_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend=backend)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard_vectors(V, rank, world, seed=3):
    """This rank's V prior vectors: disjoint slices of one seeded draw of
    V * world vectors (each replica evaluates its own vectors)."""
    from xpsi_gb300 import synthetic as SY
    return SY.config3_vectors(V * world, seed=seed)[rank * V:(rank + 1) * V]


# Instruction counts of the dominant kernel (integrate_kernel<double>), from one
# ncu capture of one launch over the first 64 prior vectors of the benchmark's
# draw (profiles/integrate_kernel_instruction_mix_64_vectors.md).  Thread
# instructions: FP64 FLOP = 2 DFMA + DMUL + DADD, FP32 FLOP = 2 FFMA + FMUL +
# FADD.  A launch over other vectors is scaled by its cost-model work (the
# kernel's own counter) relative to the captured launch's.
PIPE_COUNTS = {
    "vectors": 64,
    "cost_model_flop": 482067568128.0,
    "fp64_flop": 2 * 3645276754 + 1588912815 + 1953852419,
    "fp32_flop": 2 * 164095141825 + 58059214755 + 635536874448,
    "dram_bytes": 969295104 + 2730820608,
    "fp64_pipe_active": 0.530,
    "fma_pipe_active": 0.389,
    "issue_active": 0.547,
    "duration_ms": 68.3,
    "capture": "ncu --metrics (instruction classes, pipe activity, dram bytes) -k "
               "regex:integrate_kernel -s 1 -c 1, python bench.py --vectors 64 --steps 1 "
               "--warmup 3 --legs none",
}


def bench_config(V):
    """The workload description both arms print (identical by construction)."""
    return {"workload": WORKLOAD, "vectors_per_gpu": V,
            "vectors": "config3_vectors(V, seed=3): the first V prior draws of seed 3 "
                       "(sharded by rank under torchrun)",
            "l2": "inputs and ray tables larger than L2 (129 MB) every step"}


def gpu_data(model, device):
    """Counts drawn from the GPU's model of the full-size configuration's
    vector (the GPU arm).  The reference arm draws them from the oracle's
    model of the same vector; the two expected-count sets agree to ~1e-12, so
    the seeded Poisson draws are the same counts (checked in
    tests/test_gpu_full_size.py)."""
    import torch
    from xpsi_gb300 import batch as BT
    from xpsi_gb300 import synthetic as SY
    ev = BT.BatchEvaluator(model, device=device)
    P0 = BT.prepare(model, SY.config2_vector(seed=1)[None, :])
    B0 = ev.upload(P0)
    ev.run(B0)
    torch.cuda.synchronize()
    folded = B0["folded"].cpu().numpy()
    SY.attach_data(model, [folded[0], folded[1]], P0.shifts[0])
    return model


def oracle_data(model, n_threads):
    """Counts drawn from the oracle's model of the full-size configuration's
    vector (the reference arm)."""
    from oracle import pipeline as OP
    from oracle import prepare as OPR
    from xpsi_gb300 import synthetic as SY
    P0 = OPR.prepare(model, SY.config2_vector(seed=1)[None, :], n_threads=n_threads)
    _, _, stages = OP.loglike(model, P0, n_threads=n_threads, return_stages=True)
    SY.attach_data(model, [stages[0]["folded"], stages[1]["folded"]], P0.shifts[0])
    return model


# ------------------------------------------------------------------ GPU arm
def run_gb300(args):
    import torch
    from xpsi_gb300 import batch as BT
    rank, world = dist_init()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    V = args.vectors
    cores = os.cpu_count() or 1
    model, _ = build_workload(1)
    gpu_data(model, local)
    ev = BT.BatchEvaluator(model, device=local)
    # each rank evaluates its own V vectors (independent parameter vectors)
    params = shard_vectors(V, rank, world)
    t0 = time.time()
    P = BT.prepare(model, params)
    t_mesh = time.time() - t0
    # resident copies of the batch, the steps rotating over one CUDA stream
    # each: one batch's FP64-bound stages run beside another's FP32-bound
    # integrator sums
    from xpsi_gb300.serving import estimate_bytes
    per_batch = estimate_bytes(ev, P)
    n_res = max(1, min(args.resident, int((150 << 30) // max(1, per_batch))))
    Bs = [ev.upload(P) for _ in range(n_res)]
    B = Bs[0]
    streams = [torch.cuda.Stream() for _ in Bs]
    flops = torch.zeros(1, dtype=torch.float64, device="cuda")
    # warm-up
    pipelined_steps(ev, Bs, streams, args.warmup)
    torch.cuda.synchronize()
    # the integrator alone on one stream (CUDA events on the launching
    # stream) and its cost-model work for one step
    probe = {"flops": flops}
    ev.run(B, probe=probe)
    torch.cuda.synchronize()
    int_ms = probe["start"].elapsed_time(probe["end"])
    int_flops = float(flops.item())
    one_ms = single_stream_step(ev, B)
    # timed region
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    with clocks:
        ms = pipelined_steps(ev, Bs, streams, args.steps)
    barrier(world)
    ms = max_over_ranks(ms, world)
    st = ev.statuses(B)
    plain_ll = B["loglike"].cpu().numpy().copy()
    value = V * world / (ms / 1e3)
    del Bs, B
    torch.cuda.empty_cache()
    # end to end through the public API from the host parameter vectors:
    # each step prepares the batch (cell budgets and derived quantities on
    # the host), copies its mesh descriptors to the device (pinned), builds
    # the meshes on the GPU, runs the five stages and reads log L and the
    # statuses back
    Pg = BT.prepare(model, params, meshes="gpu")
    h2d = ev.h2d_bytes(Pg)
    d2h = V * (8 + 4)
    e2e_steps = max(2, min(args.steps, args.e2e_steps))
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for ll, stx in ev.loglikelihood_pipelined([params] * e2e_steps, depth=args.e2e_depth):
        pass
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_s = max_over_ranks(e2e_s, world)
    # the GPU mesh build of one batch alone (CUDA events around the upload,
    # whose launches are the mesh kernels and the descriptor copies)
    stream = torch.cuda.current_stream()
    g0 = torch.cuda.Event(enable_timing=True)
    g1 = torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    Bx = ev.upload(Pg)
    g1.record(stream)
    torch.cuda.synchronize()
    mesh_gpu_ms = g0.elapsed_time(g1)
    del Bx
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    BT.prepare(model, params, meshes="gpu")
    t_prep = time.perf_counter() - t0
    pk, pk_kind = peaks()
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded prior draws, "
        "Poisson counts from the model of the full-size configuration's vector)",
        "config": bench_config(V),
        "details": {"precision": "plain FP64 path (the drop-in's numerics), every vector "
                                 "of the batch in one launch per stage",
                    "streams": f"{n_res} copies of the batch resident, steps rotating over "
                               f"{n_res} CUDA streams (events bracket all steps)",
                    "ms_per_step_one_stream": one_ms,
                    "mesh_build_host_s": round(t_mesh, 3),
                    "mesh_build_gpu_ms": round(mesh_gpu_ms, 2),
                    "prepare_for_gpu_meshes_s": round(t_prep, 3),
                    "device_bytes_per_batch": per_batch,
                    "status_counts": {str(k): int(v) for k, v in
                                      zip(*np.unique(st, return_counts=True))}},
        "e2e": {"value": V * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": e2e_steps,
                "what": "from host parameter vectors: host cell budgets, pinned copies, GPU "
                        "meshes, the five stages, log L and statuses back to the host; "
                        f"BatchEvaluator.loglikelihood_pipelined, {args.e2e_depth} batches "
                        "in flight"},
        "gpu_launches": None,
        "clocks": clocks.summary(),
    }
    # kernels launched per step (the ncu launch list of this bench): rays 1;
    # integrator 6 (row costs, chunk plan, Num4D pre-pass and scan, the
    # integration, the ordered reduction); energy 1; fold 3 (row and column
    # splits, the double-float product); likelihood 2
    out["gpu_launches"] = args.steps * (1 + 6 + 1 + 3 + 2)
    out["roofline"] = roofline(int_ms, int_flops, V)
    if rank == 0:
        legs = set(args.legs.split(",")) if args.legs != "all" else \
            {"mixed", "drop_in", "serving", "cpu"}
        cpu = None
        if "cpu" in legs:
            cpu = cpu_baseline(args, model, params, plain_ll, st)
            out["cpu_baseline"] = cpu
        if "mixed" in legs:
            out["mixed"] = mixed_leg(model, P, plain_ll, st, args, cpu)
        if "drop_in" in legs:
            out["drop_in"] = drop_in_leg(model, P, min(V, args.drop_in_vectors))
            out["batched_vs_drop_in"] = value / out["drop_in"]["value"]
            if "mixed" in out:
                out["mixed_vs_drop_in"] = out["mixed"]["value"] / out["drop_in"]["value"]
        if "serving" in legs and args.serve_window > 0:
            out["serving"] = serving_leg(args)
        if cpu is not None:
            cpu.pop("_ll", None)
            cpu.pop("_st", None)
        print(json.dumps(out))


def single_stream_step(ev, B, reps=1):
    """ms of one step of the batch on one stream, alone (CUDA events)."""
    import torch
    s = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    for _ in range(reps):
        ev.run(B, stream=s)
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def roofline(int_ms, int_flops, V):
    """Per-pipe rates of the dominant kernel against the pipes' measured
    FMA peaks: its FP64 and FP32 arithmetic (ncu instruction counts of the
    captured launch, scaled to this launch by the cost-model work) over its
    CUDA-event duration in this run."""
    pk, pk_kind = peaks()
    p64, p32 = pipe_peak(1), pipe_peak(0)
    scale = int_flops / PIPE_COUNTS["cost_model_flop"] if int_flops > 0 else V / 64.0
    sec = int_ms / 1e3
    a64 = PIPE_COUNTS["fp64_flop"] * scale / sec / 1e12
    a32 = PIPE_COUNTS["fp32_flop"] * scale / sec / 1e12
    traffic = PIPE_COUNTS["dram_bytes"] * scale
    return {"bound": "fp64", "achieved": a64, "peak": p64, "unit": "TFLOP/s", "frac": a64 / p64,
            "traffic": traffic,
            "pipes": {"fp64": {"achieved": a64, "peak": p64, "frac": a64 / p64,
                               "pipe_active_ncu": PIPE_COUNTS["fp64_pipe_active"]},
                      "fp32": {"achieved": a32, "peak": p32, "frac": a32 / p32,
                               "pipe_active_ncu": PIPE_COUNTS["fma_pipe_active"]},
                      "issue_active_ncu": PIPE_COUNTS["issue_active"]},
            "kernel": "integrate_kernel<double>", "kernel_ms": int_ms,
            "cost_model_flop_per_launch": int_flops,
            "achieved_hbm_gbs": traffic / sec / 1e9, "hbm_peak_gbs": pk.get("hbm_gbs"),
            "hbm_peak_source": pk_kind,
            "peak_source": "measured here: FMA throughput probes of the FP64 and FP32 pipes "
                           "(MEASURED_PEAKS.json has HBM and bf16 only)",
            "counts_source": PIPE_COUNTS["capture"] + " (%d vectors; scaled by %.3f)"
                             % (PIPE_COUNTS["vectors"], scale),
            "note": "the busiest pipe is FP64 (ncu: %.0f %% of active cycles against %.0f %% "
                    "for the FMA pipe; most FP64-pipe instructions are conversions, "
                    "compares and the slab contraction); frac is its arithmetic rate over "
                    "its FMA peak; issue is %.0f %% active, the kernel latency-bound on "
                    "dependent double-float chains" % (100 * PIPE_COUNTS["fp64_pipe_active"],
                                                     100 * PIPE_COUNTS["fma_pipe_active"],
                                                     100 * PIPE_COUNTS["issue_active"])}


def pipe_peak(fp64):
    """FMA throughput of the FP64 (fp64=1) or FP32 (fp64=0) pipe on this GPU:
    8 independent FMA chains per thread, 8 CTAs of 256 threads per SM, best
    of three timed launches (CUDA events), TFLOP/s."""
    import torch
    from xpsi_gb300._native import lib
    buf = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    L = lib()
    iters = 4096 if fp64 else 65536
    L.xgpu_peak_probe(fp64, 152 * 8, 256, 64, buf.data_ptr(), st)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fl = L.xgpu_peak_probe(fp64, 152 * 8, 256, iters, buf.data_ptr(), st)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, fl / (e0.elapsed_time(e1) / 1e3) / 1e12)
    return best


def fp64_peak(device):
    return pipe_peak(1)



def pipelined_steps(ev, Bs, streams, steps):
    """Run `steps` evaluations of the resident batches Bs, step k on
    streams[k % len] with Bs[k % len]; returns ms per step from CUDA events
    recorded before the first and after the last step of every stream."""
    import torch
    cur = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(cur)
    for s in streams:
        s.wait_event(e0)
    for k in range(steps):
        s = streams[k % len(streams)]
        with torch.cuda.stream(s):
            ev.run(Bs[k % len(Bs)], stream=s)
    for s in streams:
        done = torch.cuda.Event()
        done.record(s)
        cur.wait_event(done)
    e1.record(cur)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / max(1, steps)


def mixed_leg(model, P, plain_ll, plain_st, args, cpu=None):
    """Batched mixed-precision form on the same vectors: throughput, and
    |Delta log L| against the FP64 path on every vector and against the
    oracle on the vectors the CPU leg evaluated."""
    import torch
    from xpsi_gb300 import batch as BT
    ev = BT.BatchEvaluator(model, precision="mixed")
    Bs = [ev.upload(P) for _ in range(2)]
    B = Bs[0]
    streams = [torch.cuda.Stream() for _ in Bs]
    pipelined_steps(ev, Bs, streams, 1)
    ms = pipelined_steps(ev, Bs, streams, max(2, min(args.steps, 4)))
    ll = B["loglike"].cpu().numpy()
    st = ev.statuses(B)
    del Bs, B
    torch.cuda.empty_cache()
    ok = (st == 0) & (plain_st == 0)
    d = np.abs(ll - plain_ll)[ok]
    out = {"value": P.V / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
           "precision": "FP32 atmosphere interpolation, Akima pieces and cell x phase sums; "
                        "tensor-core fold (3xTF32, FP32 accumulation); FP64 rays, knots, "
                        "energy integration and log L",
           "dlogL_vs_fp64": _dist(d),
           "status_equal": bool((st == plain_st).all())}
    if cpu is not None and cpu.get("_ll") is not None:
        n = len(cpu["_ll"])
        ok_o = (cpu["_st"] == 0) & (st[:n] == 0)
        out["dlogL_vs_oracle"] = _dist(np.abs(ll[:n] - cpu["_ll"])[ok_o])
    return out


def _dist(d):
    if d.size == 0:
        return {"vectors": 0}
    return {"median": float(np.median(d)), "p99": float(np.percentile(d, 99)),
            "max": float(d.max()), "frac_within_1e-3": float((d <= 1e-3).mean()),
            "vectors": int(d.size)}


def drop_in_leg(model, P, n_vec):
    """The plain FP64 drop-in: one parameter vector at a time through the
    module-level replacements of the reference callables (host arrays in and
    out, as X-PSI's HotRegion/Signal would call them)."""
    import math as _m
    from xpsi_gb300.cellmesh import rays as R, integrator_for_azimuthal_invariance as I
    from xpsi_gb300.tools import energy_integrator as EI
    from xpsi_gb300.likelihoods import default_background_marginalisation as DBM
    from xpsi_gb300 import instrument as INS
    N_L = model.regions[0].num_leaves
    N_R = model.regions[0].num_rays
    leaves = np.linspace(0.0, 2 * _m.pi, N_L)
    phases = 2 * _m.pi * np.linspace(0.0, 1.0, N_L)
    cph = np.linspace(0.0, 1.0, N_L)
    logE, logEd = np.log10(model.energies), np.log10(model.instrument.energy_edges)
    counts = np.asarray(model.data.counts, np.float64)
    K = counts.shape[0]
    pre = DBM.precomputation(np.asarray(model.data.counts, np.int32))
    sup = -np.ones((K, 2))
    sup[:, 0] = 0.0
    atm = model.atmosphere
    t0 = time.perf_counter()
    for v in range(n_vec):
        regs = []
        for h in range(P.H):
            mi = v * P.H + h
            mesh = P.meshes[mi]
            S = mesh.S0
            rs = slice(mesh.row_off, mesh.row_off + S)
            cs = slice(mesh.cell_off, mesh.cell_off + S * S)
            u = P.row["u"][rs].copy()
            ma = P.row["maxAlpha"][rs].copy()
            r_s = P.row["r_s"][mesh.row_off]
            t, D, CA, L, MD = R.compute_rays(1, S, r_s, u, ma, N_R)
            L -= P.row["lag_C"][rs][:, None]
            L *= P.row["lag_scale"][mesh.row_off]
            theta = np.repeat(P.row["theta0"][rs][:, None], S, axis=1)
            spec = model.regions[h]
            st, flux = I.integrate(1, 0.0, mesh.omega, r_s, mesh.inclination,
                                   P.cellArea[cs].reshape(S, S), P.row["radius"][rs], u, theta,
                                   P.phi[cs].reshape(S, S), P.params[cs].reshape(S, S, 2),
                                   P.radiates[cs].reshape(S, S), None, N_R, D, CA, L, MD,
                                   P.row["cos_gamma"][rs], model.energies, leaves, phases,
                                   atm if spec.atm_ext == 2 else (), None, spec.atm_ext, None, 0)
            if st != 0:
                break
            e = EI.energy_integrator(1, flux / P.d_sq[mi], logE, logEd)
            regs.append(INS.fold(model.instrument.matrix, e))
        if len(regs) == P.H:
            DBM.eval_marginal_likelihood(model.data.exposure, model.data.phase_edges, counts,
                                         regs, [cph] * P.H, P.shifts[v], pre, sup, 1000, 0.0,
                                         model.epsrel, model.epsilon, model.sigmas,
                                         model.llzero)
    dt = time.perf_counter() - t0
    return {"value": n_vec / dt, "unit": UNIT, "vectors": n_vec,
            "what": "one vector per call through the drop-in module functions "
                    "(host arrays, H2D/D2H per call), FP64"}


def serving_models():
    """The serving configuration's model mix: blackbody (the small plain
    configuration's kind) and Num4D (the full-size configuration's), each at
    sqrt_num_cells 32, 64, 96 (max 128) and 64 or 128 leaves; data drawn from
    each model's reference vector on the GPU."""
    import torch
    from xpsi_gb300 import batch as BT
    from xpsi_gb300 import synthetic as SY
    models = {}
    for kind in ("bb", "num4d"):
        for sq in (32, 64, 96):
            for nl in (64, 128):
                if kind == "bb":
                    w = SY.config1_workload()
                    m = BT.Model(regions=[BT.HotRegionSpec(atm_ext=1, sqrt_num_cells=sq,
                                                           min_sqrt_num_cells=10,
                                                           max_sqrt_num_cells=128,
                                                           num_leaves=nl, num_rays=512)],
                                 instrument=BT.Instrument(w["matrix"], w["input_edges"]),
                                 data=BT.Data(np.zeros((300, 32), np.int32), w["phase_edges"],
                                              w["exposure"]), num_energies=64)
                    ref = np.array([w["mass"], w["radius_km"], w["frequency"],
                                    math.cos(w["inclination"]), 1.0, w["colatitude"],
                                    w["spot_radius"], w["logT"], 0.0])
                else:
                    m = SY.config2_model(sqrt_num_cells=sq, num_leaves=nl)
                    ref = SY.config2_vector(seed=1)
                ev = BT.BatchEvaluator(m)
                P0 = BT.prepare(m, ref[None, :])
                B0 = ev.upload(P0)
                ev.run(B0)
                torch.cuda.synchronize()
                f = B0["folded"].cpu().numpy()
                SY.attach_data(m, [f[h] for h in range(P0.H)], P0.shifts[0])
                models[f"{kind}_{sq}_{nl}"] = (m, ref)
                del ev, B0
    return models


def serve_once(models, rate, window, max_batch, precision, seed, deadline=300.0):
    """Poisson arrivals at `rate` req/s for `window` s, batch sizes
    log-uniform on [1, max_batch], models drawn evenly; returns the
    serving record (all requests run to completion)."""
    from xpsi_gb300 import synthetic as SY
    from xpsi_gb300.serving import Server, poisson_stream
    names = sorted(models)
    stream = poisson_stream(rate, window, max_batch, seed=seed)
    rng = np.random.default_rng(seed)
    reqs = []
    for t, v in stream:
        name = names[rng.integers(len(names))]
        m, ref = models[name]
        if name.startswith("bb"):
            p = np.repeat(ref[None, :], v, axis=0)
            p[:, 5] = rng.uniform(0.5, 2.5, v)
            p[:, 6] = rng.uniform(0.03, 0.3, v)
            p[:, 8] = rng.uniform(0.0, 1.0, v)
        else:
            p = SY.config3_vectors(v, seed=int(rng.integers(1 << 30)))
        reqs.append((t, name, p))
    srv = Server({k: v[0] for k, v in models.items()}, hbm_budget=120 << 30, slots=4,
                 precision=precision, prep_threads=8)
    futs = []
    t0 = time.perf_counter()
    for t, name, p in reqs:
        while time.perf_counter() - t0 < t:
            time.sleep(0.0002)
        futs.append(srv.submit(name, p))
    done = 0
    for f in futs:
        left = deadline - (time.perf_counter() - t0)
        try:
            f.result(timeout=max(1.0, left))
            done += 1
        except Exception:  # noqa: BLE001 - recorded, the leg is bounded
            break
    wall = time.perf_counter() - t0
    srv.close()
    if done < len(futs):
        return {"incomplete": f"{done} of {len(futs)} requests finished within {deadline} s"}
    lat = srv.latency_percentiles()
    nv = sum(p.shape[0] for _, _, p in reqs)
    return {"p50_ms": lat["p50_ms"], "p99_ms": lat["p99_ms"], "requests": len(reqs),
            "vectors": nv, "throughput": nv / wall, "unit": UNIT, "wall_s": wall,
            "arrivals": f"Poisson {rate} req/s for {window} s, batch sizes log-uniform on "
                        f"[1, {max_batch}], {len(names)} models drawn evenly",
            "launches": srv.stats.launches, "merged_requests": srv.stats.merged_requests,
            "peak_concurrent_launches": srv.stats.peak_concurrency,
            "peak_device_bytes_admitted": srv.stats.peak_bytes, "hbm_budget_bytes": 120 << 30,
            "precision": precision}


def serving_leg(args):
    """The serving configuration: 200 req/s, batches log-uniform on [1, 4096]
    (about 490 vectors per request), an even blackbody / Num4D mix over
    sqrt_num_cells {32, 64, 96} x leaves {64, 128}, a 120 GB admission
    budget, plain FP64 form (the form that meets |dlogL| <= 1e-3), over a
    fixed arrival window.  It offers ~1e5 vectors/s, far beyond one GPU, so
    latencies are queue-bound and the throughput is the saturation rate.
    Beside it, a load one GPU sustains (40 req/s, batches 1-16)."""
    models = serving_models()
    sat = serve_once(models, args.serve_rate, args.serve_window, args.serve_max_batch,
                     "plain", seed=5)
    sat["what"] = "saturation: the serving configuration's arrival process over a fixed window"
    sus = serve_once(models, 40.0, 2.0, 16, "plain", seed=6)
    sus["what"] = "sustainable load"
    return {"saturation": sat, "sustainable": sus}


# ------------------------------------------------------------------ CPU legs
def oracle_evals(model, params, n_threads, budget_s, start=0):
    """The oracle over successive vectors (from `start`) until the time
    budget is used, each from its parameter vector: the oracle's own
    preparation (cell budgets and meshes included) and every restated
    stage; returns (log L [n], status [n], seconds)."""
    from oracle import pipeline as OP
    from oracle import prepare as OPR
    lls, sts, t_total = [], [], 0.0
    for v in range(start, params.shape[0]):
        t0 = time.perf_counter()
        P = OPR.prepare(model, params[v:v + 1], n_threads=n_threads)
        ll, st = OP.loglike(model, P, n_threads=n_threads)
        t_total += time.perf_counter() - t0
        lls.append(ll[0])
        sts.append(st[0])
        if t_total >= budget_s:
            break
    return np.array(lls), np.array(sts, dtype=np.int32), t_total


def cpu_baseline(args, model, params, plain_ll=None, plain_st=None):
    """The oracle on the host cores over the first vectors of the batch, and
    |Delta log L| of the GPU's plain path against it on those vectors."""
    cores = os.cpu_count() or 1
    ll, st, t = oracle_evals(model, params, cores, args.cpu_budget)
    n = len(ll)
    out = {"value": n / t, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"the first {n} vectors of the batch through the oracle (oracle/: its "
                     f"own meshes and every restated stage, OpenMP over parallels, {cores} "
                     f"threads), {t:.1f} s", "_ll": ll, "_st": st}
    if plain_ll is not None:
        ok = (st == 0) & (plain_st[:n] == 0)
        out["plain_vs_oracle"] = {"status_equal": bool((st == plain_st[:n]).all()),
                                  **_dist(np.abs(plain_ll[:n] - ll)[ok])}
    return out


def run_reference(args):
    rank, world = dist_init()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    model, _ = build_workload(1)
    oracle_data(model, cores)
    V = args.vectors
    params = shard_vectors(V, 0, 1)
    per_step = max(1.0, args.cpu_budget / max(1, args.steps))
    for _ in range(args.warmup):
        oracle_evals(model, params[:1], cores, 0.0)
    n_tot, t_tot, v0 = 0, 0.0, 0
    for s in range(args.steps):
        ll, st, t = oracle_evals(model, params, cores, per_step, start=v0 % V)
        n_tot += len(ll)
        v0 += len(ll)
        t_tot += t
    value = n_tot / t_tot
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_tot / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded prior draws, Poisson counts from the model of the "
                   "full-size configuration's vector)",
           "config": bench_config(V),
           "impl": "reference",
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                            "sample": f"the first {n_tot} vectors of the batch through the "
                                      f"oracle (its own meshes and every restated stage; "
                                      f"OpenMP, {cores} threads), about {per_step:.1f} s per "
                                      f"step"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def _cpu_worker(args):
    """One single-threaded oracle process over its share of the vectors for
    `seconds`: (evaluations, seconds)."""
    model_kind, params, seconds = args
    sys.path.insert(0, HERE)
    from xpsi_gb300 import synthetic as SY
    model = SY.config2_model() if model_kind == 2 else SY.config1_model()
    if model_kind == 2:
        oracle_data(model, 1)
    else:
        _oracle_data_config1(model, 1)
    n, t = 0, 0.0
    for v in range(params.shape[0]):
        ll, st, dt = oracle_evals(model, params[v:v + 1], 1, 0.0)
        n += 1
        t += dt
        if t >= seconds:
            break
    return n, t


def _oracle_data_config1(model, n_threads):
    from oracle import pipeline as OP
    from oracle import prepare as OPR
    from xpsi_gb300 import synthetic as SY
    P0 = OPR.prepare(model, SY.config1_vector()[None, :], n_threads=n_threads)
    _, _, stages = OP.loglike(model, P0, n_threads=n_threads, return_stages=True)
    SY.attach_data(model, [stages[0]["folded"]], P0.shifts[0])
    return model


def run_cpu_configs(args):
    """The reference path's CPU cost per configuration through the oracle
    (meshes included) on this host: latency (one process on all cores,
    median of repeated evaluations of the configuration's vector) and
    throughput (one single-threaded process per core over distinct prior
    vectors)."""
    import multiprocessing as mp
    from xpsi_gb300 import synthetic as SY
    cores = os.cpu_count() or 1
    out = {"cores": cores, "kind": "port (oracle/, its own meshes and every restated stage)"}
    for kind in (1, 2):
        model = SY.config1_model() if kind == 1 else SY.config2_model()
        vec = SY.config1_vector() if kind == 1 else SY.config2_vector(seed=1)
        (_oracle_data_config1 if kind == 1 else oracle_data)(model, cores)
        lat = []
        for _ in range(args.cpu_reps):
            _, _, t = oracle_evals(model, vec[None, :], cores, 0.0)
            lat.append(t)
        if kind == 1:
            rng = np.random.default_rng(3)
            prm = np.repeat(vec[None, :], 64 * cores, axis=0)
            prm[:, 5] = rng.uniform(0.5, 2.5, prm.shape[0])
            prm[:, 6] = rng.uniform(0.03, 0.3, prm.shape[0])
        else:
            prm = SY.config3_vectors(64 * cores, seed=3)
        shares = [(kind, prm[c::cores], args.cpu_budget) for c in range(cores)]
        with mp.get_context("spawn").Pool(cores) as pool:
            res = pool.map(_cpu_worker, shares)
        n = sum(r[0] for r in res)
        thr = sum(r[0] / r[1] for r in res if r[1] > 0)
        out[f"config{kind}"] = {"latency_s_median": statistics.median(lat),
                                "latency_samples": len(lat), "throughput_evals_per_s": thr,
                                "throughput_evaluations": n,
                                "throughput_vectors": "config 1: the vector with spot colatitude "
                                "U(0.5, 2.5) and radius U(0.03, 0.3)" if kind == 1 else
                                "config 3's prior draws (seed 3)"}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    # the batched configuration: 4096 prior vectors in one launch
    ap.add_argument("--vectors", type=int, default=4096)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    # comma-separated subset of mixed,drop_in,serving,cpu (or "all", "none"):
    # the legs run after the timed plain-path steps
    ap.add_argument("--legs", default="all")
    ap.add_argument("--resident", type=int, default=2,
                    help="copies of the batch resident for the timed steps (one stream each)")
    ap.add_argument("--e2e-depth", type=int, default=2,
                    help="batches in flight in the end-to-end leg")
    ap.add_argument("--e2e-steps", type=int, default=4)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--drop-in-vectors", type=int, default=64)
    # the serving configuration: Poisson arrivals at 200 req/s, batches
    # log-uniform on [1, 4096], over a fixed arrival window
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-window", type=float, default=0.1)
    ap.add_argument("--serve-max-batch", type=int, default=4096)
    # per-configuration CPU latency and throughput of the reference path
    # (oracle) on this host, instead of the benchmark
    ap.add_argument("--cpu-configs", action="store_true")
    ap.add_argument("--cpu-reps", type=int, default=5)
    args = ap.parse_args()
    if args.cpu_configs:
        run_cpu_configs(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
