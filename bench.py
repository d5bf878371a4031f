#!/usr/bin/env python
"""Benchmark of the gravity forward path (prism model, mixed precision).

Workload: the mixed-precision forward of a 256x256x64 prism mesh
(1 x 1 x 0.5 km cells, seeded Gaussian density +- 300 kg/m^3 plus 20 box
anomalies) at 128x128 stations draped on seeded fractal topography
(0-3 km): 6.87e10 (station, prism) pairs per step.  A step is one full
forward (all pairs) with the inputs resident in HBM.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Our arm prints value = pairs/s over all ranks (weak scaling: every rank
runs the full workload; no collective on the data path), e2e = the same
through the public API with pinned host buffers (H2D of density and
stations and D2H of gz inside the timed region), the roofline of the
dominant kernel against the measured FP32 FMA issue peak, and the CPU
baseline (the double-precision oracle on the host cores, bounded sample).
The reference arm times the reference's own CPU gravity code (the lambda
of TFM.cpp:95-99, point mass in double, compiled from TFM.cpp by
oracle/build.py) on the host cores, on the same geometry, on a bounded
sample of station rows and nodes.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "prism·station gz evals/s and gradient evals/s; mixed vs FP64 at ≤1e-6 rel err"
UNIT = "evals/s"
WORKLOAD = ("mixed-precision prism forward, 256x256x64 prisms (1x1x0.5 km), 128x128 stations "
            "draped on fractal topography 0-3 km")
# Executed float flops per evaluated (station, prism) slot of the far kernel,
# by form (FMA = 2; the rsqrt on the special-function unit is not a flop),
# counted from prism_common.cuh / prism.cu per lane of the packed operations:
#   sixth order (far_unit2): Z 2, r^2 2, u 1, Horner 6 FMA 12, three products 3,
#     density accumulate 2 -> 22
#   second order (far_unit2_t2): Z 2, r^2 2, u 1, two FMA 4, three products 3,
#     accumulate 2 -> 14
#   column pairs: second order with one Z for two columns -> 13
# plus the compensation step per 32 slots (an add and a 4-operation Kahan
# update: 5/32).  The slot counts come from the counting variant of the same
# kernel, run once per bench (ztm_ctx_count_forms), so that the numerator is
# the work this launch executes.
FLOPS_PER_SLOT = {"sixth_order": 22 + 5 / 32, "second_order": 14 + 5 / 32,
                  "column_pairs": 13 + 5 / 32}
# DRAM bytes of one far_kernel launch on this workload, ncu
# dram__bytes_read.sum + dram__bytes_write.sum (the capture and its command
# are in profiles/prism_far_256x256x64_draped.md)
FAR_TRAFFIC_BYTES = 26.4e6
L2_BYTES = 129 * 2 ** 20


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def max_over_ranks(dist, x):
    """The largest x of all ranks (a host float), through the process
    group's own backend: a device tensor for NCCL, a host tensor for gloo."""
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline_prism(mesh, rho, st, nsample=224):
    import numpy as np
    import oracle
    idx = np.linspace(0, len(st) - 1, nsample).astype(int)
    t0 = time.perf_counter()
    oracle.prism_mesh(mesh, rho, st[idx])
    dt = time.perf_counter() - t0
    pairs = nsample * mesh.nx * mesh.ny * mesh.nz
    return {"value": pairs / dt, "unit": UNIT, "cores": oracle.NTHREADS, "kind": "port",
            "sample": "%d of %d stations x all %d prisms, closed form in double (oracle/oracle.c)"
                      % (nsample, len(st), mesh.nx * mesh.ny * mesh.nz), "seconds": dt}


def run_reference(args, rank):
    """The reference's own CPU gravity code (TFM.cpp:95-99: the GFM lambda,
    cut verbatim out of TFM.cpp and compiled with g++ -O3 into
    oracle/_ref/libref_tfm.so) on the host cores, one std::thread per
    station row as TFM.cpp:99 launches it, on the same geometry mapped onto
    its node grid.  A step is a bounded sample: as many station rows as the
    host has cores, each over every 16th selected node (the per-pair work is
    that of the full sum)."""
    if rank != 0:
        return 0
    import numpy as np
    import oracle
    from ztm_gb300 import synth
    mesh, rho, st = synth.draped_mesh_256x256x64()
    g, drho, surf = synth.pointmass_grid_of_mesh(mesh, rho, st)
    nn_all = np.nonzero(np.abs(drho) > g.threshold)[0].astype(np.int32)
    stride = int(os.environ.get("ZTM_REF_NODE_STRIDE", "16"))
    nn = np.ascontiguousarray(nn_all[::stride])
    rows = max(1, min(g.dj, os.cpu_count() or 1))
    if oracle.ref_tfm_available():
        kind, algo = "reference", ("the reference's own GFM lambda (TFM.cpp:95-99, point mass in "
                                   "double) cut verbatim out of TFM.cpp and compiled with g++ -O3 "
                                   "(oracle/_ref/libref_tfm.so); one thread per station row")

        def sample():
            oracle.ref_tfm_rows(g, drho, surf, 0, rows, nn=nn)
    else:  # no reference sources and no generated harness: the restatement
        kind, algo = "port", ("TFM.cpp:95-99 restated operation for operation in oracle/oracle.c "
                              "(bit-identical to the compiled lambda where both exist)")

        def sample():
            oracle.pointmass_tfm_sample(g, drho, surf, 0, rows * g.di, nn=nn, nthreads=rows)
    times = []
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        sample()
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
    pairs = rows * g.di * nn.size
    value = pairs * len(times) / sum(times)
    smp = ("%d station rows x %d stations x %d of the %d selected nodes (every %dth) per step"
           % (rows, g.di, nn.size, nn_all.size, stride))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(args.gpus),
            "algorithm": algo + "; same geometry as our arm on the reference's node grid "
                                "(h = 1 km, fv = 2)",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": rows, "kind": kind,
                             "sample": smp},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def config_dict(n):
    return {"workload": WORKLOAD, "prisms": [256, 256, 64], "cell_m": [1000, 1000, 500],
            "stations": [128, 128], "pairs_per_step": 256 * 256 * 64 * 128 * 128,
            "precision": "mixed: far pairs float (sixth-order expansion, second order beyond 48 "
                         "half-diagonals, compensated sums), near region and per-station sums "
                         "double", "near_q": 4,
            "l2": "flushed between timed steps (256 MiB write)",
            "parallelism": "replica per GPU" if n > 1 else "single GPU"}


def run_ours(args, rank, local_rank, world):
    import numpy as np
    import torch
    import ztm_gb300
    from ztm_gb300 import synth
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    ctx = ztm_gb300.GravityContext(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    mesh, rho, st = synth.draped_mesh_256x256x64()
    np_ = mesh.nx * mesh.ny * mesh.nz
    pairs = np_ * len(st)
    d_rho = torch.tensor(rho, device="cuda")
    d_st = torch.tensor(st, device="cuda")
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device="cuda")

    def step():
        return ctx.prism(mesh, d_rho, d_st, precision="mixed")

    for _ in range(args.warmup):
        step()
    # one untimed step of the counting variant: the slots of each form
    ctx.count_forms(True)
    step()
    ctx.sync()
    forms = ctx.form_counts()
    ctx.count_forms(False)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    clocks = ClockSampler(local_rank) if rank == 0 else None
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = ctx.launches()
    ctx.profile(True)
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()  # L2 flush, outside the step's events
        ev[i][0].record(stream)
        out = step()
        ev[i][1].record(stream)
    ctx.sync()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop() if clocks else None
    launches = ctx.launches() - launches0
    far_ms, far_n = ctx.profile_read("prism_far")
    ctx.profile(False)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_s = sum(step_ms) / 1e3
    if dist:
        total_s = max_over_ranks(dist, total_s)
    value = world * pairs * args.steps / total_s
    ms_per_step = 1e3 * total_s / args.steps
    gz = out.cpu().numpy()
    if not np.all(np.isfinite(gz)):
        raise RuntimeError("non-finite gz")

    # end to end through the public API: pinned host buffers, H2D+D2H inside
    h_rho = torch.empty(np_, dtype=torch.float64, pin_memory=True).numpy()
    h_rho[:] = rho
    h_st = torch.empty(st.size, dtype=torch.float64, pin_memory=True).numpy().reshape(-1, 3)
    h_st[:] = st
    e2e_steps = max(1, min(args.steps, 5))
    ctx.prism(mesh, h_rho, h_st, precision="mixed")
    e2e_t = []
    for _ in range(e2e_steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        ctx.sync()
        t0 = time.perf_counter()
        g_host = ctx.prism(mesh, h_rho, h_st, precision="mixed")
        e2e_t.append(time.perf_counter() - t0)
    e2e_total = max_over_ranks(dist, sum(e2e_t)) if dist else sum(e2e_t)
    e2e = {"value": world * pairs * e2e_steps / e2e_total, "unit": UNIT,
           "h2d_bytes_per_step": int(h_rho.nbytes + h_st.nbytes),
           "d2h_bytes_per_step": int(g_host.nbytes)}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    peak32 = ctx.measure_peak("fp32")
    far_avg = far_ms / max(far_n, 1)
    slots = dict(zip(("sixth_order", "second_order", "column_pairs"), forms[:3]))
    flops = sum(slots[f] * FLOPS_PER_SLOT[f] for f in slots)
    achieved = flops / (far_avg * 1e-3) / 1e12
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": config_dict(world), "clocks": clk, "e2e": e2e,
            "gpu_launches": launches,
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak32,
                         "unit": "TFLOP/s", "frac": achieved / peak32 if peak32 else None,
                         "traffic": FAR_TRAFFIC_BYTES,
                         "kernel": "far_kernel: far fields (FMA pipe) and near regions "
                                   "(FP64 pipe) in one persistent grid",
                         "flops_per_launch": flops, "slots_per_launch": slots,
                         "flops_per_slot": FLOPS_PER_SLOT,
                         "near_phi_per_launch": forms[3],
                         "pairs_per_launch": pairs, "kernel_ms": far_avg,
                         "algorithmic_bytes_per_launch": np_ * 4 + len(st) * 32,
                         "traffic_source": "ncu dram bytes read + written, one launch "
                                           "(profiles/prism_far_256x256x64_draped.md)",
                         "peak_source": "measured FP32 FMA issue rate on this GPU "
                                        "(ztm_measure_peak; MEASURED_PEAKS.json has only HBM "
                                        "and bf16 tensor peaks, neither bounds this kernel)"},
            "kernels_ms": {"far_kernel": far_avg, "step": ms_per_step}}
    if not args.quick:
        line.update(extras(ctx, mesh, rho, st, d_rho, d_st, gz, ms_per_step))
        if world == 1:
            line["cpu_baseline"] = cpu_baseline_prism(mesh, rho, st)
            line["other_workloads"] = other_workloads(ctx)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def _median_ms(ctx, fn, n):
    """Median device time of n replays of fn (one warm-up call first), CUDA
    events on the context's stream around each replay."""
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream)
    out = fn()
    ctx.sync()
    ms = []
    for _ in range(n):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        ctx.sync()
        ms.append(e0.elapsed_time(e1))
    return statistics.median(ms), out


FIELD_FIXTURE = os.path.join(ROOT, "tests", "golden", "prism_256x256x64_draped_fp64.npz")


def full_field_accuracy(rho, st, gz_mixed):
    """The mixed field at every station against the committed double field
    of the same inputs (tests/golden/make_prism_field.py: the CPU oracle,
    every prism at every station)."""
    import numpy as np
    if not os.path.exists(FIELD_FIXTURE):
        return None
    z = np.load(FIELD_FIXTURE)
    same = (abs(float(np.sum(rho)) - float(z["rho_sum"])) <= 1e-9 * float(z["rho_abs_sum"]) and
            np.allclose(rho[::9973], z["rho_sample"], rtol=0, atol=1e-9) and
            np.allclose(np.sum(st, axis=0), z["st_sum"], rtol=1e-12))
    if not same:
        return {"error": "inputs differ from the fixture's fingerprint"}
    ref = z["gz"]
    err = np.abs(gz_mixed - ref)
    rel = err / np.abs(ref)
    return {"stations": int(ref.size), "normwise_rel_err": float(err.max() / np.abs(ref).max()),
            "max_station_rel_err": float(rel.max()), "p99_station_rel_err":
            float(np.percentile(rel, 99)), "reference": "double-precision CPU oracle, all stations"}


def extras(ctx, mesh, rho, st, d_rho, d_st, gz_mixed, fwd_ms):
    """Side measurements: the mixed field against the double field at every
    station, the plain FP64 kernel's rate, gradient evals/s of the adjoint,
    the reference's point-mass model on the same geometry (ours and the
    reference GF kernel itself).  Rates are medians of replays."""
    import numpy as np
    import torch
    import oracle
    from ztm_gb300 import synth
    out = {}
    np_ = mesh.nx * mesh.ny * mesh.nz
    acc = full_field_accuracy(rho, st, gz_mixed)
    if acc is not None:
        out["accuracy_full_field"] = acc
    sub = np.arange(0, len(st), len(st) // 64)[:64]
    ds = torch.tensor(st[sub], device="cuda")
    ms64, ref = _median_ms(ctx, lambda: ctx.prism(mesh, d_rho, ds, precision="fp64"), 10)
    r = ref.cpu().numpy()
    m = gz_mixed[sub]
    out["fp64_plain"] = {"value": np_ * len(sub) / (ms64 * 1e-3), "unit": UNIT,
                         "sample": "%d stations x all prisms, median of 10" % len(sub)}
    out["accuracy"] = {"normwise_rel_err_vs_fp64": float(np.max(np.abs(m - r)) / np.max(np.abs(r))),
                       "max_station_rel_err": float(np.max(np.abs(m - r) / np.abs(r))),
                       "stations_checked": len(sub), "reference": "the plain FP64 GPU kernel"}
    # gradient evals/s: adjoint of the same forward (d misfit / d rho)
    res = torch.tensor(np.random.default_rng(0).normal(0, 1, len(st)), device="cuda")
    msa, _ = _median_ms(ctx, lambda: ctx.adjoint(mesh, d_st, res, precision="mixed"), 10)
    out["gradient"] = {"value": np_ * len(st) / (msa * 1e-3), "unit": "gradient evals/s",
                       "ms": msa, "what": "d misfit / d rho, all pairs, mixed, median of 10"}
    rs = torch.tensor(np.random.default_rng(0).normal(0, 1, len(sub)), device="cuda")
    msa64, _ = _median_ms(ctx, lambda: ctx.adjoint(mesh, ds, rs, precision="fp64"), 10)
    out["fp64_plain_adjoint"] = {"value": np_ * len(sub) / (msa64 * 1e-3),
                                 "unit": "gradient evals/s",
                                 "sample": "%d stations x all prisms, median of 10" % len(sub)}
    pairs = np_ * len(st)
    t64 = pairs / out["fp64_plain"]["value"] + pairs / out["fp64_plain_adjoint"]["value"]
    tmx = (fwd_ms + msa) * 1e-3
    out["forward_plus_adjoint_vs_plain_fp64"] = {
        "mixed_s": tmx, "fp64_s_at_measured_rates": t64, "speedup": t64 / tmx,
        "what": "mixed forward (the timed step) + mixed adjoint against the plain double forward "
                "+ adjoint of the same pairs at their measured rates (vertex-shared double kernels)"}
    # the reference's own point-mass model on the same geometry (its grid,
    # every node as a station): our float and double gathers and adjoints
    g, drho, surf = synth.pointmass_grid_of_mesh(mesh, rho, st)
    nodes32 = int(np.count_nonzero(np.abs(drho.astype(np.float32)) > 0.001))
    nodes64 = int(np.count_nonzero(np.abs(drho) > 0.001))
    dd, dsf = torch.tensor(drho, device="cuda"), torch.tensor(surf, device="cuda")
    dw = torch.tensor(np.random.default_rng(1).normal(0, 1, g.di * g.dj), device="cuda")
    pm = {}
    for prec, nodes, n in (("fp32", nodes32, 10), ("fp64", nodes64, 3)):
        ms, _ = _median_ms(ctx, lambda: ctx.pointmass(g, dd, dsf, precision=prec), n)
        msj, _ = _median_ms(ctx, lambda: ctx.pointmass_adjoint(g, dsf, dw, drho=dd,
                                                               precision=prec), n)
        pm[prec] = {"value": nodes * mesh.nx * mesh.ny / (ms * 1e-3), "unit": "point-mass pairs/s",
                    "ms": ms, "adjoint_value": nodes64 * mesh.nx * mesh.ny / (msj * 1e-3),
                    "adjoint_ms": msj, "replays": n}
    out["pointmass_gpu"] = pm
    if oracle.ref_gf_available():
        gf, ms = oracle.ref_gf(g, drho.astype(np.float32), surf.astype(np.float32), reps=3)
        out["reference_gf_gpu"] = {
            "value": nodes32 * mesh.nx * mesh.ny / (ms * 1e-3), "unit": "point-mass pairs/s",
            "ms": ms, "what": "reference GF kernel (GFM_GPU.cu:16-22) compiled unchanged for "
                              "sm_103a, same geometry on its grid (%d stations x %d nodes), mean "
                              "of 3 launches" % (mesh.nx * mesh.ny, nodes32)}
    return out


def _timed(ctx, fn, reps=1):
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream)
    fn()
    ctx.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        out = fn()
    e1.record(stream)
    ctx.sync()
    return e0.elapsed_time(e1) / reps, out


def other_workloads(ctx):
    """The other workloads (interface adjoint, line-search batch, LM steps,
    interface inversion), not the headline: calls under a second timed as the
    median of 10 replays, the double interface call and the inversions
    once."""
    import numpy as np
    import torch
    from ztm_gb300 import synth
    res = {}
    # adjoint workload: 256x256 interface columns, 128x128 stations
    im, depth, rho, st, start = synth.moho_columns()
    rng = np.random.default_rng(3)
    d = lambda a: torch.tensor(a, device="cuda")
    dd, dr, ds, d0 = d(depth), d(rho), d(st), d(start)
    data = ctx.interface(im, dd, dr, ds, precision="fp64")
    ctx.sync()
    data = data + d(rng.normal(0, 0.05, len(st)))
    ms_m, out_m = _median_ms(ctx, lambda: ctx.interface_misfit(im, d0, dr, ds, data,
                                                             precision="mixed"), 10)
    ms_d, out_d = _timed(ctx, lambda: ctx.interface_misfit(im, d0, dr, ds, data, precision="fp64"))
    pairs = im.nx * im.ny * len(st)
    err = lambda a, b: float((a - b).abs().max() / b.abs().max())
    res["adjoint_interface_256x256"] = {
        "pairs": pairs, "mixed_ms_forward_plus_adjoint": ms_m, "fp64_ms_forward_plus_adjoint": ms_d,
        "speedup_vs_fp64": ms_d / ms_m,
        "mixed_gz_evals_plus_gradient_evals_per_s": 2 * pairs / (ms_m * 1e-3),
        "rel_err_vs_fp64": {"misfit": float(abs(out_m[0] - out_d[0]) / out_d[0]),
                            "gz": err(out_m[1], out_d[1]), "g_rho": err(out_m[2], out_d[2]),
                            "g_depth": err(out_m[3], out_d[3])}}
    # batched workload: 32 line-search trials + 16 uneven regional meshes
    jobs, alphas = synth.line_search_batch()
    djobs = [(m_, d(r_.reshape(r_.shape[0], -1) if r_.ndim == 2 else r_), d(s_)) for m_, r_, s_ in jobs]
    ctx.batch(djobs)  # builds and caches the graph
    ctx.sync()
    ms_b, outs = _median_ms(ctx, lambda: ctx.batch(djobs), 10)
    mp = sum(int(r_.shape[0]) * m_.nx * m_.ny * m_.nz * len(s_) for m_, r_, s_ in jobs)
    one = ctx.prism(jobs[0][0], djobs[0][1][5], djobs[0][2], precision="mixed")
    ctx.sync()
    res["batched_32_trials_plus_16_meshes"] = {
        "model_pairs": mp, "ms": ms_b, "model_pair_evals_per_s": mp / (ms_b * 1e-3),
        "launches_per_call": "1 graph: 4 prep kernels and a library station sort per job + 1 persistent kernel",
        "rel_err_trial5_vs_single_call": err(outs[0][5], one)}
    # the damped Gauss-Newton trials of LMA::fit (TFM.cpp:159-160): the GPU at
    # the reference's size, and against the reference's own zmath code (the
    # CPU baseline: MTM, inv and the products, compiled unchanged) at 600
    # parameters x 3000 data, 4 damping pairs
    import oracle
    rng = np.random.default_rng(7)
    dm = np.array([[0.0, 0.0], [1e-3, 1e-4], [0.1, 1e-2], [1.0, 1.0]])
    lm = {}
    for nrows, ncols in ((3000, 600), (12000, 2700)):
        J = rng.normal(size=(nrows, ncols)) * rng.uniform(0.1, 10.0, ncols)[None, :]
        r_, b_, sg = rng.normal(size=nrows), rng.normal(size=ncols), rng.uniform(0.05, 2.0, ncols)
        dJ, dr_, db_, ds_, ddm = d(J), d(r_), d(b_), d(sg), d(dm)
        ms, B = _median_ms(ctx, lambda: ctx.lm_steps(dJ, dr_, db_, ds_, ddm), 10)
        row = {"gpu_ms": ms, "damping_pairs": 4, "replays": "median of 10"}
        if ncols == 600 and oracle.ref_lm_available():
            t0 = time.perf_counter()
            Bref, _ = oracle.ref_lm_steps(J, r_, b_, sg, dm)
            row["reference_cpu_s"] = time.perf_counter() - t0
            row["reference"] = ("zmath.cpp compiled unchanged + TFM.cpp:159-160 (MTM with one "
                                "thread per column, inv per damping pair on its own thread)")
            step = Bref - b_[None, :]
            row["rel_diff_steps"] = float(np.max(np.abs((B.cpu().numpy() - b_[None, :]) - step)) /
                                          np.max(np.abs(step)))
            row["speedup"] = row["reference_cpu_s"] / (ms * 1e-3)
        lm["J_%dx%d" % (nrows, ncols)] = row
    res["lm_steps"] = lm
    # inversion workload: 512x512 columns, 256x256 stations, 20 L-BFGS iterations
    im5, dep5, rho5, st5, start5 = synth.moho_columns_512()
    data5 = ctx.interface(im5, d(dep5), d(rho5), d(st5), precision="fp64")
    ctx.sync()
    data5 = data5.cpu().numpy() + np.random.default_rng(5).normal(0, 0.05, len(st5))
    t0 = time.perf_counter()
    dep_out, hist, nit = ctx.invert_interface(im5, start5, rho5, st5, data5, lam=1e-2, iterations=20,
                                              precision="mixed")
    dt = time.perf_counter() - t0
    res["inversion_512x512_20_iterations"] = {
        "method": "L-BFGS", "seconds": dt, "iterations": nit, "misfit_start": float(hist[0]),
        "misfit_end": float(hist[-1]), "pairs_per_forward": im5.nx * im5.ny * len(st5),
        "mean_abs_depth_error_m": {"start": float(np.abs(start5 - dep5).mean()),
                                   "end": float(np.abs(dep_out - dep5).mean())}}
    t0 = time.perf_counter()
    dep_gn, hist_gn, nit_gn = ctx.invert_interface(im5, start5, rho5, st5, data5, lam=1e-2,
                                                   iterations=20, precision="mixed", method="gn",
                                                   cg_iterations=10)
    dt = time.perf_counter() - t0
    res["inversion_512x512_20_iterations_gauss_newton"] = {
        "method": "Gauss-Newton, 10 CG steps (J v + J^T w) per iteration", "seconds": dt,
        "iterations": nit_gn, "misfit": [float(x) for x in hist_gn],
        "noise_floor_misfit": 0.5 * len(st5) * 0.05 ** 2,
        "mean_abs_depth_error_m": {"start": float(np.abs(start5 - dep5).mean()),
                                   "end": float(np.abs(dep_gn - dep5).mean())}}
    return res


def inversion_study(ctx, fp64_iterations=3):
    """The interface inversion workload (512x512 columns of 0.5 km, 256x256
    stations, lambda = 1e-2) against double precision: data from the plain
    double forward of the true Moho plus 0.05 mGal noise; the mixed L-BFGS
    run of 20 iterations; its final model's misfit re-evaluated with the
    double forward; and the first iterations of the same inversion run in
    plain double beside it (each double evaluation is a full forward and
    adjoint over 1.7e10 pairs).  Prints one JSON line."""
    import numpy as np
    from ztm_gb300 import synth
    im, dep, rho, st, start = synth.moho_columns_512()
    t0 = time.perf_counter()
    data = ctx.interface(im, dep, rho, st, precision="fp64")
    t_data = time.perf_counter() - t0
    data = data + np.random.default_rng(5).normal(0, 0.05, len(st))
    t0 = time.perf_counter()
    dm, hm, nm = ctx.invert_interface(im, start, rho, st, data, lam=1e-2, iterations=20,
                                      precision="mixed")
    t_mixed = time.perf_counter() - t0
    t0 = time.perf_counter()
    mis64_final = 0.5 * float(np.sum((ctx.interface(im, dm, rho, st, precision="fp64") - data) ** 2))
    t_check = time.perf_counter() - t0
    t0 = time.perf_counter()
    dd, hd, nd = ctx.invert_interface(im, start, rho, st, data, lam=1e-2,
                                      iterations=fp64_iterations, precision="fp64")
    t_fp64 = time.perf_counter() - t0
    k = min(len(hd), len(hm))
    noise_floor = 0.5 * len(st) * 0.05 ** 2
    line = {"workload": "inversion", "what": __doc_line__(inversion_study),
            "columns": im.nx * im.ny, "stations": len(st), "lambda": 1e-2,
            "data": "plain double forward of the true model + N(0, 0.05 mGal)",
            "mixed": {"iterations": nm, "seconds": t_mixed, "misfit": [float(x) for x in hm],
                      "mean_abs_depth_error_m": float(np.abs(dm - dep).mean())},
            "final_model_misfit_fp64": mis64_final,
            "final_model_misfit_mixed": float(hm[-1]),
            "final_misfit_rel_diff": abs(mis64_final - float(hm[-1])) / mis64_final,
            "fp64": {"iterations": nd, "seconds": t_fp64, "misfit": [float(x) for x in hd],
                     "mean_abs_depth_error_m": float(np.abs(dd - dep).mean())},
            "trajectory_max_rel_diff_first_%d" % k:
                float(np.max(np.abs(np.asarray(hm[:k]) - np.asarray(hd[:k])) / np.asarray(hd[:k]))),
            "noise_floor_misfit": noise_floor,
            "start_mean_abs_depth_error_m": float(np.abs(start - dep).mean()),
            "seconds_fp64_forward": t_data, "seconds_fp64_check": t_check}
    print(json.dumps(line), flush=True)
    return 0


def __doc_line__(f):
    return " ".join(f.__doc__.split())


def run_workload(args, local_rank):
    """The other workloads as the timed step (side measurements and ncu
    targets; the default forward workload is the headline)."""
    import numpy as np
    import torch
    import ztm_gb300
    from ztm_gb300 import synth
    torch.cuda.set_device(local_rank)
    ctx = ztm_gb300.GravityContext(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    d = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    if args.workload == "adjoint":
        mesh, rho, st = synth.draped_mesh_256x256x64()
        ds = d(st)
        res = d(np.random.default_rng(0).normal(0, 1, len(st)))
        units = mesh.nx * mesh.ny * mesh.nz * len(st)
        what = "d misfit/d rho of the 256x256x64 mesh at 128x128 stations (gradient evals)"
        step = lambda: ctx.adjoint(mesh, ds, res, precision="mixed")
    elif args.workload == "interface":
        im, depth, rho, st, start = synth.moho_columns()
        dd, dr, dst, d0 = d(depth), d(rho), d(st), d(start)
        data = ctx.interface(im, dd, dr, dst, precision="fp64")
        ctx.sync()
        units = 2 * im.nx * im.ny * len(st)
        what = ("forward + adjoint (misfit, d/drho, d/ddepth) of 256x256 Moho columns at "
                "128x128 stations (gz evals + gradient evals)")
        step = lambda: ctx.interface_misfit(im, d0, dr, dst, data, precision="mixed")
    elif args.workload in ("batch", "batch_tuned"):
        jobs, _ = synth.line_search_batch()
        djobs = [(m_, d(r_), d(s_)) for m_, r_, s_ in jobs]
        if args.workload == "batch_tuned":  # every candidate shape and variant, timed once
            ctx.batch(djobs, autotune=True)
            ctx.sync()
            print(json.dumps({"batch_tuning": ctx.tuning(),
                              "columns": ["stage_kb", "log2_pairs_per_item", "variant", "us"]}),
                  flush=True)
        units = sum(int(r_.shape[0]) * m_.nx * m_.ny * m_.nz * len(s_) for m_, r_, s_ in jobs)
        what = ("32 line-search trials on the 256x256x64 mesh + 16 regional meshes, one "
                "graph-captured persistent launch (model-pair evals)")
        step = lambda: ctx.batch(djobs)
    elif args.workload == "batch_trials_small":
        jobs, _ = synth.line_search_batch(n_regional=0)
        mesh, trials, st = jobs[0]
        sub = np.ascontiguousarray(st[::8])
        djobs = [(mesh, d(trials), d(sub))]
        ctx.batch(djobs, autotune=True)  # every candidate shape and variant, timed once
        ctx.sync()
        print(json.dumps({"batch_tuning": ctx.tuning(),
                          "columns": ["stage_kb", "log2_pairs_per_item", "variant", "us"]}),
              flush=True)
        units = int(trials.shape[0]) * mesh.nx * mesh.ny * mesh.nz * len(sub)
        what = ("32 line-search trials on the 256x256x64 mesh at every 8th station (2,048), "
                "the fastest shape: the profiling case of the batched kernel (model-pair evals)")
        step = lambda: ctx.batch(djobs, autotune=True)
    elif args.workload == "pointmass":
        mesh, rho, st = synth.draped_mesh_256x256x64()
        g, drho, surf = synth.pointmass_grid_of_mesh(mesh, rho, st)
        dd, dsf = d(drho), d(surf)
        units = int(np.count_nonzero(np.abs(drho.astype(np.float32)) > 0.001)) * mesh.nx * mesh.ny
        what = ("the reference's point-mass model (float) on the 256x256x64 draped-mesh geometry, its grid: "
                "every node a station (pairs of selected nodes x stations)")
        step = lambda: ctx.pointmass(g, dd, dsf, precision="fp32")
    elif args.workload in ("pointmass_adjoint", "pointmass_adjoint64"):
        mesh, rho, st = synth.draped_mesh_256x256x64()
        g, drho, surf = synth.pointmass_grid_of_mesh(mesh, rho, st)
        dd, dsf = d(drho), d(surf)
        dw = d(np.random.default_rng(0).normal(0, 1, g.di * g.dj))
        prec = "fp64" if args.workload.endswith("64") else "fp32"
        sel = np.abs(drho) > 0.001
        units = int(np.count_nonzero(sel)) * g.di * g.dj
        what = ("transposed point-mass sum (%s) on the 256x256x64 draped-mesh geometry, its grid: "
                "selected nodes x stations" % prec)
        step = lambda: ctx.pointmass_adjoint(g, dsf, dw, drho=dd, precision=prec)
    elif args.workload == "forward_small":
        mesh, rho, st = synth.draped_mesh_256x256x64()
        sub = np.ascontiguousarray(st[::8])
        dr, ds = d(rho), d(sub)
        units = mesh.nx * mesh.ny * mesh.nz * len(sub)
        what = ("mixed prism forward of the 256x256x64 draped mesh at every 8th of its stations "
                "(2,048): the profiling case of the far kernel")
        step = lambda: ctx.prism(mesh, dr, ds, precision="mixed")
    elif args.workload == "prism_f64":
        mesh, rho, st = synth.draped_mesh_256x256x64()
        sub = st[np.arange(0, len(st), len(st) // 64)[:64]]
        dr, ds = d(rho), d(sub)
        units = mesh.nx * mesh.ny * mesh.nz * len(sub)
        what = ("plain double prism forward (vertex-shared) of the 256x256x64 draped mesh at 64 of "
                "its stations")
        step = lambda: ctx.prism(mesh, dr, ds, precision="fp64")
    elif args.workload in ("pointmass_small", "pointmass64_small", "pointmass_adjoint_small",
                           "pointmass_adjoint64_small"):
        # the 128x128 top-left columns and 32 top layers of the draped mesh on
        # the reference grid: 128x128 stations x 5.4e5 nodes
        mesh, rho, st = synth.draped_mesh_256x256x64()
        r3 = rho.reshape(64, 256, 256)[:32, :128, :128]
        m2 = ztm_gb300.make_mesh(128, 128, 32, mesh.dx, mesh.dy, mesh.dz)
        st2 = st[(st[:, 0] < 128 * mesh.dx) & (st[:, 1] < 128 * mesh.dy)]
        g, drho, surf = synth.pointmass_grid_of_mesh(m2, np.ascontiguousarray(r3).ravel(), st2)
        dd, dsf = d(drho), d(surf)
        prec = "fp64" if "64" in args.workload else "fp32"
        units = int(np.count_nonzero(np.abs(drho) > 0.001)) * g.di * g.dj
        if "adjoint" in args.workload:
            dw = d(np.random.default_rng(0).normal(0, 1, g.di * g.dj))
            what = "transposed point-mass sum (%s), 128x128x33-node grid, every node a station" % prec
            step = lambda: ctx.pointmass_adjoint(g, dsf, dw, drho=dd, precision=prec)
        else:
            what = "point-mass forward (%s), 128x128x33-node grid, every node a station" % prec
            step = lambda: ctx.pointmass(g, dd, dsf, precision=prec)
    elif args.workload == "lm":
        rng = np.random.default_rng(0)
        nrows, ncols, nd = 12000, 2700, 4
        J = rng.normal(size=(nrows, ncols)) * rng.uniform(0.1, 10.0, ncols)[None, :]
        dJ, dr_, db = d(J), d(rng.normal(size=nrows)), d(rng.normal(size=ncols))
        dsig = d(rng.uniform(0.05, 2.0, ncols))
        dm = d(np.array([[0.0, 0.0], [1e-3, 1e-4], [0.1, 1e-2], [1.0, 1.0]]))
        # units: the multiply-adds of J^T J (full) and of a Gauss-Jordan inversion
        # per pair (the reference's work); the library factorises by blocked LU
        units = nrows * ncols * ncols + nd * ncols ** 3
        what = ("damped Gauss-Newton trials (TFM.cpp:159-160): J 12000 x 2700, 4 damping pairs "
                "(J^T J + 4 solves by blocked LU; units: the multiply-adds of J^T J and of the "
                "reference's Gauss-Jordan inversions)")
        step = lambda: ctx.lm_steps(dJ, dr_, db, dsig, dm)
    elif args.workload == "inversion":
        return inversion_study(ctx)
    else:
        raise SystemExit("unknown workload " + args.workload)
    for _ in range(args.warmup):
        step()
    ctx.sync()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    for i in range(args.steps):
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    ctx.sync()
    ms = sum(a.elapsed_time(b) for a, b in ev) / args.steps
    print(json.dumps({"workload": args.workload, "what": what, "value": units / (ms * 1e-3),
                      "unit": "evals/s", "ms_per_step": ms, "steps": args.steps,
                      "warmup": args.warmup, "evals_per_step": units}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--quick", action="store_true", help="skip side measurements")
    ap.add_argument("--workload", default="forward",
                    choices=["forward", "adjoint", "interface", "batch", "pointmass",
                             "pointmass_adjoint", "pointmass_adjoint64", "inversion",
                             "prism_f64", "forward_small", "pointmass_small", "batch_tuned", "pointmass64_small",
                             "pointmass_adjoint_small", "pointmass_adjoint64_small", "lm",
                             "batch_trials_small"],
                    help="forward (the headline) or another workload as the timed step")
    args = ap.parse_args()
    rank, local_rank, world = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank)
    if args.workload != "forward":
        return run_workload(args, local_rank)
    return run_ours(args, rank, local_rank, world)


if __name__ == "__main__":
    sys.exit(main())
