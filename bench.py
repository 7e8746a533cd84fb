#!/usr/bin/env python3
"""Benchmark of the ERT forward operator + Jacobian on GB300.

One step = one Gauss-Newton iteration's operator work: ``response(model)``
(assembly, SR right-hand sides, multi-RHS PCG over all current sources,
collect, apparent resistivities) followed by ``createJacobian(model)``
(dense D x P Jacobian), on a seeded synthetic workload (default
``box_3d_large``: 256 electrodes on 16 x 16, 7392 data, 806,760 tetrahedra,
144,648 nodes).  The headline form is the mixed-precision block PCG with the
learned preconditioner (packaged weights) to an FP64 true relative residual
of 1e-10, with an FP32 Jacobian built from FP64-exact potential differences;
the plain FP64 Jacobi block PCG (FP64 Jacobian) and the FSAI form are timed
beside it on the same workload, and the three forms on ``box_3d`` (96
electrodes, 5336 data, 485,640 tetrahedra) in ``box_3d_forms``.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``value`` is device time per step with the inputs resident in HBM (CUDA
events around K steps on the launching stream).  ``e2e`` is the same step
through the reference-facing C ABI with host buffers (ertgb_response_host,
ertgb_jacobian_host): the model copied in, the apparent resistivities and the
full Jacobian copied out.  ``complex_form`` and ``cem_form`` time complex
resistivity and the total-potential operator with complete-electrode-model
patches on ``box_3d``.  ``cpu_baseline`` and ``--impl reference`` time the
CPU oracle port (the reference's algorithm restated in numpy/scipy with a
SuperLU direct solve) on bounded samples of the workload (one core beside the
GPU timings, resp. every host thread); ``--impl reference --ref-cpp`` times
full steps of the reference's own C++ where its library was built.  ``--case`` runs single workloads for
profiler captures.  With N > 1 ranks (torchrun) every rank runs an
independent replica of the workload (the operator uses one GPU).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fwd+Jacobian s/GN-iter: learned-precond vs plain GPU PCG @1e-6; %HBM peak"
UNIT = "s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["box_3d", "box_3d_probe", "box_3d_coarse", "box_3d_large",
                                           "box_3d_large_p2", "line_2d"],
                    default="box_3d_large")
    ap.add_argument("--rtol", type=float, default=1e-10)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    ap.add_argument("--precond", choices=["jacobi", "fsai", "learned", "ic0", "band"], default="learned")
    ap.add_argument("--weights", default=None, help="learned preconditioner weights (.npz); default: the "
                    "packaged weights trained for the workload")
    ap.add_argument("--no-plain", action="store_true", help="skip the comparison runs (plain FP64 Jacobi, FSAI)")
    ap.add_argument("--cem-only", action="store_true", help="with --no-plain: still time the CEM form")
    ap.add_argument("--cem-patch", type=float, default=4.0 / 3.0,
                    help="surface cell size of the workload mesh (CEM patch = the triangles within one diagonal)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-cpp", action="store_true",
                    help="with --impl reference: time full steps of the reference's own C++ "
                         "(oracle/_ref/libgimli_ref.so, present only where the reference's sources were "
                         "compiled) instead of the sampled port")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--gn", action="store_true", help="also time one full Gauss-Newton iteration per form "
                    "(response, Jacobian, 200 CGLS iterations on the GPU, line-search responses)")
    ap.add_argument("--case", choices=["complex", "refine", "jacobian", "batch", "gn2d"], default=None,
                    help="run one single workload for a profiler instead of the bench and print one line: "
                    "'complex' = one complex-resistivity response + complex Jacobian (-10 mrad, --precision), "
                    "'refine' = the GPU H2 refinement of the workload mesh, twice, "
                    "'jacobian' = one response (--precision, --precond) and three Jacobians (FP32 with "
                    "--precision mixed, else FP64), "
                    "'batch' = the batched 2.5-D configuration (--batch-problems of the 64 seeded problems, "
                    "21 explicit wavenumbers each): batched responses (mixed; FP64 side by side) against the "
                    "same problems' responses one after another (mixed and plain FP64), "
                    "'gn2d' = one Gauss-Newton iteration per solver form on the largest of those meshes")
    ap.add_argument("--batch-problems", type=int, default=64)
    return ap.parse_args()


def run_batch_case(args):
    """The batched 2.5-D configuration: seeded problems of 2k-60k nodes with
    24-72 electrodes (dipole-dipole + Wenner), 21 explicit wavenumbers each
    (setkValues / setWeights: 17 Gauss-Legendre + 4 Gauss-Laguerre points
    over each problem's electrode distances), one batched mixed-precision
    response against the same problems solved one after another."""
    import torch
    from pygimli_gb300 import synthetic
    from pygimli_gb300.batch import BatchedERTModelling
    from pygimli_gb300.ert import ERTModelling
    from pygimli_gb300.kwave import kwave_list
    probs = synthetic.batch_2d(64)[:args.batch_problems]

    def fop_for(mesh, data, precision, precond="jacobi"):
        p = data.sensorPositions()
        d = np.linalg.norm(p[:, None, :] - p[None, :, :], axis=2)
        k, w = kwave_list(d[d > 0].min() / 2.0, d.max() * 2.0, 17, 4)
        f = ERTModelling(precision=precision, precond=precond, rtol=args.rtol, maxIter=200000)
        f.setkValues(k)
        f.setWeights(w)
        f.setData(data)
        f.setMesh(mesh, ignoreRegionManager=True)
        return f

    models = [r for _, _, r in probs]
    rec = {"case": "batch", "problems": len(probs), "wavenumbers": 21,
           "nodes": [int(m.nodeCount()) for m, _, _ in probs],
           "rhs_columns": int(sum(21 * d.sensorCount() for _, d, _ in probs))}
    batch = BatchedERTModelling([fop_for(m, d, "mixed") for m, d, _ in probs])
    for label in ("batched_mixed_first_s", "batched_mixed_s"):  # the first call also tunes the tile shape
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out_b = batch.response(models)
        torch.cuda.synchronize()
        rec[label] = time.perf_counter() - t0
    rec["batch_info"] = {k: v for k, v in (batch.info or {}).items() if not isinstance(v, list)}
    del batch
    torch.cuda.empty_cache()
    # the same problems in FP64: their FP64 solves side by side (one stream each)
    batch64 = BatchedERTModelling([fop_for(m, d, "fp64") for m, d, _ in probs])
    for label in ("batched_fp64_first_s", "batched_fp64_s"):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out_b64 = batch64.response(models)
        torch.cuda.synchronize()
        rec[label] = time.perf_counter() - t0
    del batch64
    torch.cuda.empty_cache()
    # the banded direct solve (exact Cholesky per wavenumber): batched and one after another
    batchb = BatchedERTModelling([fop_for(m, d, "fp64", "band") for m, d, _ in probs])
    for label in ("batched_band_first_s", "batched_band_s"):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out_bb = batchb.response(models)
        torch.cuda.synchronize()
        rec[label] = time.perf_counter() - t0
    del batchb
    torch.cuda.empty_cache()
    t_seq = 0.0
    for m, d, r in probs:
        f = fop_for(m, d, "fp64", "band")
        f.response(r)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f.response(r)
        torch.cuda.synchronize()
        t_seq += time.perf_counter() - t0
        del f
    rec["sequential_band_s"] = t_seq
    rec["max_rel_diff_rhoa_band_vs_fp64_pcg"] = float(max(np.max(np.abs(np.asarray(a) - np.asarray(b)) /
                                                                 np.asarray(b)) for a, b in zip(out_bb, out_b64)))
    for precision in ("mixed", "fp64"):
        t_seq, dev = 0.0, 0.0
        for (m, d, r), rb in zip(probs, out_b):
            f = fop_for(m, d, precision)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rs = f.response(r)
            torch.cuda.synchronize()
            t_seq += time.perf_counter() - t0
            dev = max(dev, float(np.max(np.abs(np.asarray(rb) - rs) / rs)))
            del f
        rec[f"sequential_{precision}_s"] = t_seq
        rec[f"max_rel_diff_rhoa_batched_vs_sequential_{precision}"] = dev
    rec["ratio_sequential_mixed_to_batched"] = rec["sequential_mixed_s"] / rec["batched_mixed_s"]
    rec["ratio_sequential_fp64_to_batched_fp64"] = rec["sequential_fp64_s"] / rec["batched_fp64_s"]
    rec["ratio_sequential_band_to_batched_band"] = rec["sequential_band_s"] / rec["batched_band_s"]
    rec["ratio_sequential_fp64_pcg_to_batched_band"] = rec["sequential_fp64_s"] / rec["batched_band_s"]
    rec["max_rel_diff_rhoa_batched_fp64_vs_mixed"] = float(max(np.max(np.abs(np.asarray(a) - np.asarray(b)) / np.asarray(b))
                                                               for a, b in zip(out_b, out_b64)))
    print(json.dumps(rec), flush=True)


def run_gn2d_case(args):
    """One Gauss-Newton iteration (response, Jacobian, CGLS, line search) on
    the largest mesh of the batched 2.5-D configuration's first 16 problems
    (21 explicit wavenumbers), per solver form: the banded direct solve, the
    plain FP64 PCG (Jacobi, IC(0)) and the mixed-precision PCG with the learned
    preconditioner (line_2d weights) and with FSAI.  Observed data = the
    model's response with 2 % noise; start = homogeneous median model."""
    import torch
    from pygimli_gb300 import synthetic
    from pygimli_gb300.ert import ERTModelling
    from pygimli_gb300.inversion import GaussNewton
    from pygimli_gb300.kwave import kwave_list
    probs = synthetic.batch_2d(64)[:16]
    mesh, data, rho = max(probs, key=lambda t: t[0].nodeCount())
    p = data.sensorPositions()
    d = np.linalg.norm(p[:, None, :] - p[None, :, :], axis=2)
    k, w = kwave_list(d[d > 0].min() / 2.0, d.max() * 2.0, 17, 4)
    forms = {"band_direct_fp64": dict(precision="fp64", precond="band"),
             "jacobi_fp64": dict(precision="fp64", precond="jacobi"),
             "ic0_fp64": dict(precision="fp64", precond="ic0"),
             "learned_mixed": dict(precision="mixed", precond="learned", weights=default_weights("line_2d")),
             "fsai_mixed": dict(precision="mixed", precond="fsai")}
    rec = {"case": "gn2d", "nodes": int(mesh.nodeCount()), "cells": int(mesh.cellCount()), "data": int(data.size()),
           "electrodes": int(data.sensorCount()), "wavenumbers": 21}
    obs = None
    for name, f in forms.items():
        fop = ERTModelling(rtol=args.rtol, maxIter=200000, **f)
        fop.setkValues(k)
        fop.setWeights(w)
        fop.setData(data)
        fop.setMesh(mesh, ignoreRegionManager=True)
        if obs is None:
            obs = fop.response(rho) * (1.0 + 0.02 * np.random.default_rng(3).normal(size=data.size()))
        gn = GaussNewton(fop, obs, np.full(data.size(), 0.02), lam=20.0)
        model = np.full(mesh.cellCount(), float(np.median(obs)))
        resp = fop.response(model)
        gn.step(model, resp)  # warm-up (allocations, graph capture, band ordering)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        resp = fop.response(model)
        its = fop.stats()["iterations"]
        _, _, info = gn.step(model, resp)
        torch.cuda.synchronize()
        rec[name] = {"value": time.perf_counter() - t0, "unit": "s", "pcg_iterations_first_response": its,
                     "cgls_iterations": info["cgls_iterations"], "forward_responses": info["responses"] + 1,
                     "phi_before": info["phi_before"], "phi_after": info["phi_after"]}
        del fop, gn
        torch.cuda.empty_cache()
    print(json.dumps(rec), flush=True)


def run_case(args):
    """One single workload (``--case``) for ``ncu`` launch lists and captures."""
    import torch
    from pygimli_gb300 import build as _build
    _build.build()
    if args.case == "batch":
        run_batch_case(args)
        return
    if args.case == "gn2d":
        run_gn2d_case(args)
        return
    mesh, data, rho, _ = workload(args.workload)
    if args.case == "refine":
        from pygimli_gb300 import refine
        for _ in range(2):
            t0 = time.perf_counter()
            h = refine.createH2(mesh, 0)
        print(f"refine {args.workload}: H2 of {mesh.cellCount()} cells -> {h.cellCount()} in "
              f"{time.perf_counter() - t0:.4f} s")
        return
    from pygimli_gb300.ert import ERTModelling
    if args.case == "jacobian":
        weights = (args.weights or default_weights(args.workload)) if args.precond == "learned" else None
        fop = ERTModelling(precision=args.precision, precond=args.precond, weights=weights)
        fop.setData(data)
        fop.setMesh(mesh, ignoreRegionManager=True)
        fop.response(rho)
        ms = []
        for _ in range(3):
            J = fop.createJacobian(rho, dtype="float32" if args.precision == "mixed" else "float64")
            ms.append(fop.stats()["ms_jacobian"])
            del J
        print(f"jacobian {args.workload} {args.precision}: {data.size()} x {fop.parameterCount} J, "
              f"ms per launch {', '.join(f'{x:.3f}' for x in ms)}")
        return
    fop = ERTModelling(precision=args.precision)
    fop.setData(data)
    fop.setMesh(mesh, ignoreRegionManager=True)
    fop.setComplex(True)
    z = rho * np.exp(-0.01j)
    t0 = time.perf_counter()
    fop.response(z)
    fop.createJacobian(z)
    torch.cuda.synchronize()
    st = fop.stats()
    print(f"complex {args.workload} {args.precision}: {time.perf_counter() - t0:.3f} s, COCG iterations "
          f"{st['iterations']}, columns finished in FP64 {st['stalled_columns']}")


def workload_label(name, mesh, data, rho=None):
    if name == "line_2d":
        return (f"line_2d: 2.5-D, 41 electrodes, 741 dipole-dipole, {mesh.nodeCount()} nodes, "
                f"{mesh.cellCount()} triangles, 17 wavenumbers")
    ne = "256 electrodes (16x16 @4 m)" if name.startswith("box_3d_large") else "96 electrodes (12x8 @4 m)"
    order = "P2" if name.endswith("p2") else "P1"
    return (f"{name}: 3-D, {ne}, {data.size()} ABMN, {mesh.nodeCount()} nodes, {mesh.cellCount()} tetrahedra, "
            f"{order}")


def workload(name):
    from pygimli_gb300 import synthetic
    if name == "line_2d":
        mesh, data, rho = synthetic.line_2d()
    elif name.startswith("box_3d_large"):
        mesh, data, rho = synthetic.box_3d_large(p2=name.endswith("p2"))
    else:
        # box_3d_coarse: the box_3d scheme on a para mesh of 4 m cells (124k
        # tetrahedra, a 2.6 GB FP32 Jacobian) for profiler captures
        mesh, data, rho = synthetic.box_3d(scheme="inline" if name == "box_3d_probe" else "full",
                                           **({"h": 4.0} if name == "box_3d_coarse" else {}))
    return mesh, data, rho, {"workload": workload_label(name, mesh, data, rho)}


def default_weights(name):
    """Packaged weights trained on the workload's kind of matrix (element order
    and dimension): box_3d for every P1 3-D workload, box_3d_p2 for P2."""
    if name.startswith("box_3d"):
        base = "box_3d_p2" if name.endswith("p2") else "box_3d"
    else:
        base = name
    return os.path.join(ROOT, "pygimli_gb300", "weights", base + ".npz")


def dist_init(n):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if n > 0 else "gloo")
    return world, rank, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.p = None
        # let nvidia-smi finish its start-up (first sample written) before the
        # timed region begins, so that its initialisation does not overlap it
        t_end = time.perf_counter() + 3.0
        while self.p is not None and self.p.poll() is None and time.perf_counter() < t_end:
            if os.path.getsize(self.f.name) > 0:
                break
            time.sleep(0.02)

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return float("nan")

        sm = np.array([num(r[1]) for r in rows])
        mx = np.array([num(r[2]) for r in rows])
        power = np.array([num(r[3]) for r in rows])
        loaded = power >= np.nanpercentile(power, 50) if np.isfinite(power).any() else np.ones(len(rows), bool)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = [nm for i, nm in enumerate(names) if any(r[5 + i].lower().startswith("active") for r in rows)]
        return {"sm_mhz": float(np.nanmedian(sm[loaded])), "sm_max_mhz": float(np.nanmax(mx)),
                "samples": len(rows), "reasons": reasons}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel_file):
    """DRAM bytes per launch from a committed ncu summary (profiles/*.txt,
    line ``dram_bytes_per_launch = <bytes>``), else None."""
    p = os.path.join(ROOT, "profiles", kernel_file)
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        for line in fh:
            if line.strip().startswith("dram_bytes_per_launch"):
                try:
                    return float(line.split("=")[1].split()[0])
                except (IndexError, ValueError):
                    return None
    return None


def max_over_ranks(ms, world, device=None):
    """The slowest rank's time (the job ends when the last replica does):
    all-reduce MAX over the process group (NCCL on GPUs, gloo on CPU)."""
    if world <= 1:
        return float(ms)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, world, rank):
    """The reference's CPU algorithm for the path (the oracle port: the
    reference's own C++ needs its sources, which are not on the machine that
    runs the benchmark) on the same workload with every host thread.  Each of
    the K steps runs a bounded sample: the factorization is timed once (in
    the first step) and charged to every step, the Jacobian's per-electrode
    products run over all cells every step, 16 source solves and 64 Jacobian
    rows are sampled per step and scaled (oracle/cpu_baseline.py)."""
    if rank != 0:
        return
    if args.ref_cpp:
        run_reference_cpp(args)
        return
    from oracle.cpu_baseline import SampledBaseline, host_threads
    from pygimli_gb300.kwave import init_kwave_list
    mesh, data, rho, cfg = workload(args.workload)
    k, w = init_kwave_list(mesh.dim(), data.sensorPositions())
    base = SampledBaseline(mesh, data, k, w)
    threads = host_threads()
    for _ in range(max(1, min(args.warmup, 1))):  # light warm-up: one assembly
        base.P.assemble(rho, 0)
    times, descs, walls = [], [], []
    for i in range(args.steps):
        t0 = time.perf_counter()
        t, desc = base.step(rho, n_src=16, n_rows=64, threads=threads, seed=i)
        walls.append(time.perf_counter() - t0)
        times.append(t)
        descs.append(desc)
    value = float(np.mean(times))
    sample = (descs[-1] + f"; {len(times)} steps, sample wall {walls[0]:.1f} s (first step, with the "
              f"factorization) then {np.mean(walls[1:]) if len(walls) > 1 else 0.0:.1f} s per step")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": len(times),
           "warmup": args.warmup, "ms_per_step": value * 1e3,
           "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded)", "impl": "reference",
           "config": dict(cfg, parallelism="cpu", solver="SuperLU direct (CHOLMOD stand-in)"),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_reference_cpp(args):
    """Full steps (response + createJacobian, no sampling) of the reference's
    own DCSRMultiElectrodeModelling compiled from its sources
    (oracle/_ref/libgimli_ref.so), with every host thread
    (setThreadCount) and SciPy's SuperLU as the stand-in for CHOLMOD
    (the reference's setSolver hook).  The Jacobian stays in the
    reference's FP64 RMatrix."""
    from oracle import ref_driver
    from oracle.cpu_baseline import host_threads
    if not ref_driver.available():
        raise SystemExit("--ref-cpp: oracle/_ref/libgimli_ref.so is not built here "
                         "(make -C oracle needs the reference's sources)")
    mesh, data, rho, cfg = workload(args.workload)
    threads = host_threads()
    t0 = time.perf_counter()
    R = ref_driver.RefModelling(mesh, data.sensorPositions(), data.abmn(), data["k"], threads=threads, sr=True)
    setup_s = time.perf_counter() - t0
    times, resp = [], []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        R.response(rho)
        t1 = time.perf_counter()
        shape = R.create_jacobian(rho)
        t2 = time.perf_counter()
        if i >= args.warmup:
            times.append(t2 - t0)
            resp.append(t1 - t0)
    R.close()
    value = float(np.mean(times))
    sample = (f"full steps of the reference's C++ (DCSRMultiElectrodeModelling, {threads} threads, SuperLU "
              f"stand-in for CHOLMOD): response {np.mean(resp):.2f} s + createJacobian "
              f"{value - np.mean(resp):.2f} s ({shape[0]} x {shape[1]} FP64); setup {setup_s:.1f} s")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": len(times),
           "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
           "config": dict(cfg, parallelism="cpu", solver="SuperLU direct (CHOLMOD stand-in)"),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "reference", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def gn_iteration(args, mesh, data, rho, local, weights):
    """Wall time of one Gauss-Newton iteration through the public API for the
    headline form and the plain FP64 form: synthetic observations = response
    of the workload model with 2 % noise, start = homogeneous median model."""
    import torch
    from pygimli_gb300.ert import ERTModelling
    from pygimli_gb300.inversion import GaussNewton
    out = {}
    forms = {"headline": dict(precision=args.precision, precond=args.precond, weights=weights,
                              jdt="float64" if args.precision == "fp64" else "float32"),
             "plain_fp64": dict(precision="fp64", precond="jacobi", weights=None, jdt="float64")}
    obs = None
    for name, f in forms.items():
        fop = ERTModelling(device=local, rtol=args.rtol, precision=f["precision"], precond=f["precond"],
                           weights=f["weights"])
        fop.setData(data)
        fop.setMesh(mesh, ignoreRegionManager=True)
        if obs is None:
            obs = fop.response(rho) * (1.0 + 0.02 * np.random.default_rng(3).normal(size=data.size()))
        gn = GaussNewton(fop, obs, np.full(data.size(), 0.02), lam=20.0, jacobian_dtype=f["jdt"])
        model = np.full(mesh.cellCount(), float(np.median(obs)))
        resp = fop.response(model)
        gn.step(model, resp)  # warm-up (allocations, graph capture)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        resp = fop.response(model)
        pcg_first = fop.stats()["iterations"]
        _, _, info = gn.step(model, resp)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out[name] = {"value": dt, "unit": UNIT, "pcg_iterations_first_response": pcg_first,
                     "cgls_iterations": info["cgls_iterations"], "tau": info["tau"],
                     "forward_responses": info["responses"] + 1, "phi_before": info["phi_before"],
                     "phi_after": info["phi_after"]}
        del fop, gn
        torch.cuda.empty_cache()
    out["ratio_plain_to_headline"] = out["plain_fp64"]["value"] / out["headline"]["value"]
    return out


def _cpu_baseline_worker(name, n_src, n_rows, q):
    """CPU baseline in its own (spawned) process: the oracle port on one host
    core, on a bounded sample of the workload (oracle/cpu_baseline.py)."""
    sys.path.insert(0, ROOT)
    from oracle.cpu_baseline import SampledBaseline
    from pygimli_gb300.kwave import init_kwave_list
    try:
        mesh, data, rho, _ = workload(name)
        k, w = init_kwave_list(mesh.dim(), data.sensorPositions())
        base = SampledBaseline(mesh, data, k, w)
        t0 = time.perf_counter()
        t, desc = base.step(rho, n_src=n_src, n_rows=n_rows, threads=1)
        q.put({"value": t, "desc": desc, "wall_s": time.perf_counter() - t0})
    except Exception as exc:  # reported in the bench line
        q.put({"error": f"{type(exc).__name__}: {exc}"})


def run_ours(args, world, rank, local):
    cpu_q = cpu_p = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the CPU baseline runs on one host core beside the GPU timings (it needs
        # no GPU); started before CUDA is initialised, in a spawned process
        import multiprocessing as mp
        ctx = mp.get_context("spawn")
        cpu_q = ctx.Queue()
        cpu_p = ctx.Process(target=_cpu_baseline_worker, args=(args.workload, 4, 32, cpu_q), daemon=True)
        cpu_p.start()
    import ctypes

    import torch
    from pygimli_gb300 import _native
    from pygimli_gb300 import build as _build
    from pygimli_gb300.ert import ERTModelling
    _build.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = _native.load()
    mesh, data, rho, cfg = workload(args.workload)
    t_setup = time.perf_counter()
    weights = None
    if args.precond == "learned":
        weights = args.weights or default_weights(args.workload)
    fop = ERTModelling(device=local, rtol=args.rtol, precision=args.precision, precond=args.precond,
                       weights=weights)
    fop.setData(data)
    fop.setMesh(mesh, ignoreRegionManager=True)
    setup_s = time.perf_counter() - t_setup
    D, P, C = data.size(), fop.parameterCount, mesh.cellCount()
    rho_d = torch.from_numpy(rho).to(dev)
    rhoa_d = torch.empty(D, dtype=torch.float64, device=dev)
    jdt = 0 if args.precision == "fp64" else 1
    J_d = torch.empty((D, P), dtype=torch.float64 if jdt == 0 else torch.float32, device=dev)

    def step():
        fop._response_dev(rho_d, rhoa_d)
        stream = torch.cuda.current_stream(dev).cuda_stream
        fop._check(L.ertgb_jacobian(fop._ctx, ctypes.c_void_p(rho_d.data_ptr()), C,
                                    ctypes.c_void_p(J_d.data_ptr()), jdt, ctypes.c_void_p(stream)))

    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    clocks = Clocks(int(os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[0])
                    if os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].isdigit() else local)
    # one event between consecutive steps: recording adds no synchronisation,
    # and the per-step durations show whether a single step is an outlier
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    torch.cuda.synchronize()
    ev[0].record()
    for i in range(args.steps):
        step()
        ev[i + 1].record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = ev[0].elapsed_time(ev[-1])
    step_ms = [round(ev[i].elapsed_time(ev[i + 1]), 2) for i in range(args.steps)]
    st = fop.stats()
    launches = int(st["launches_response"] + st["launches_jacobian"]) * args.steps
    total_ms = max_over_ranks(total_ms, world, dev)
    value = total_ms / 1e3 / (args.steps * world)

    def time_form(wl, precision, precond, jac_dtype, label, weights_=None, n_steps=3, n_warm=2, ref_rhoa=None):
        """One step of another solver form on workload ``wl`` = (mesh, data,
        rho): CUDA events over ``n_steps`` steps after ``n_warm`` warm-up steps."""
        m_, d_, r_ = wl
        fop_p = ERTModelling(device=local, rtol=args.rtol, precision=precision, precond=precond, weights=weights_)
        fop_p.setData(d_)
        fop_p.setMesh(m_, ignoreRegionManager=True)
        Dp, Pp, Cp = d_.size(), fop_p.parameterCount, m_.cellCount()
        rp = torch.from_numpy(r_).to(dev)
        Jp = torch.empty((Dp, Pp), dtype=torch.float64 if jac_dtype == 0 else torch.float32, device=dev)
        rhoa_p = torch.empty(Dp, dtype=torch.float64, device=dev)

        def step_p():
            fop_p._response_dev(rp, rhoa_p)
            stream = torch.cuda.current_stream(dev).cuda_stream
            fop_p._check(L.ertgb_jacobian(fop_p._ctx, ctypes.c_void_p(rp.data_ptr()), Cp,
                                          ctypes.c_void_p(Jp.data_ptr()), jac_dtype, ctypes.c_void_p(stream)))

        for _ in range(n_warm):
            step_p()
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record()
        for _ in range(n_steps):
            step_p()
        f1.record()
        torch.cuda.synchronize()
        stp = fop_p.stats()
        out = {"value": f0.elapsed_time(f1) / 1e3 / n_steps, "unit": UNIT, "steps": n_steps, "solver": label,
               "jacobian": "FP64" if jac_dtype == 0 else "FP32 (FP64 differences)",
               "pcg_iterations": stp["iterations"], "ms_solve": stp["ms_solve"],
               "ms_jacobian": stp["ms_jacobian"]}
        if ref_rhoa is not None:
            out["max_rel_diff_rhoa_vs_headline_form"] = float(torch.max(torch.abs(ref_rhoa - rhoa_p) /
                                                                        torch.abs(rhoa_p)).item())
        else:
            out["rhoa"] = rhoa_p.clone()
        del Jp, fop_p
        torch.cuda.empty_cache()
        return out

    def time_cem(wl, precision, precond, jac_dtype, label):
        """The total-potential operator (ERTModelling(sr=False)) on workload
        ``wl``'s mesh with every electrode a complete-electrode-model patch
        (the surface triangles within one cell diagonal of it, contact
        impedance 1 Ohm m^2): one extension row per electrode; response +
        Jacobian, 1 warm-up and 1 timed step."""
        from pygimli_gb300.cem import mark_cem_electrodes
        m_, d_, r_ = wl
        h = float(args.cem_patch)
        mesh_c = mark_cem_electrodes(m_, d_.sensorPositions()[:, :2], h * np.sqrt(2.0) * (1.0 + 1e-6))
        fop_c = ERTModelling(sr=False, device=local, rtol=args.rtol, precision=precision, precond=precond)
        fop_c.setData(d_)
        fop_c.setMesh(mesh_c, ignoreRegionManager=True)
        Dc, Pc, Cc = d_.size(), fop_c.parameterCount, m_.cellCount()
        rc = torch.from_numpy(r_).to(dev)
        Jc = torch.empty((Dc, Pc), dtype=torch.float64 if jac_dtype == 0 else torch.float32, device=dev)
        out_c = torch.empty(Dc, dtype=torch.float64, device=dev)

        def step_c():
            fop_c._response_dev(rc, out_c)
            stream = torch.cuda.current_stream(dev).cuda_stream
            fop_c._check(L.ertgb_jacobian(fop_c._ctx, ctypes.c_void_p(rc.data_ptr()), Cc,
                                          ctypes.c_void_p(Jc.data_ptr()), jac_dtype, ctypes.c_void_p(stream)))

        step_c()
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record()
        step_c()
        f1.record()
        torch.cuda.synchronize()
        stc = fop_c.stats()
        e = fop_c._electrodes
        res = {"value": f0.elapsed_time(f1) / 1e3, "unit": UNIT, "steps": 1, "solver": label,
               "electrodes": "CEM", "extension_rows": int(e.n_ext), "extension_entries": int(len(e.rows)),
               "pcg_iterations": stc["iterations"], "ms_solve": stc["ms_solve"], "ms_jacobian": stc["ms_jacobian"],
               "columns_finished_fp64": stc["stalled_columns"],
               "jacobian": "FP64" if jac_dtype == 0 else "FP32 (FP64 differences)"}
        del Jc, fop_c
        torch.cuda.empty_cache()
        return res

    def time_complex(wl, precision):
        """Complex resistivity (IP) on workload ``wl``: the reference's
        total-potential complex formulation, block COCG + complex Jacobian;
        phases of -10 mrad on the workload's amplitudes."""
        m_, d_, r_ = wl
        fop_c = ERTModelling(device=local, rtol=args.rtol, precision=precision)
        fop_c.setData(d_)
        fop_c.setMesh(m_, ignoreRegionManager=True)
        fop_c.setComplex(True)
        Dc, Cc = d_.size(), m_.cellCount()
        zr = torch.from_numpy(r_ * np.cos(-0.01)).to(dev)
        zi = torch.from_numpy(r_ * np.sin(-0.01)).to(dev)
        out_c = torch.empty((2, Dc), dtype=torch.float64, device=dev)
        Jc = torch.empty((Dc, fop_c.parameterCount), dtype=torch.complex128, device=dev)

        def step_c():
            stream = torch.cuda.current_stream(dev).cuda_stream
            fop_c._check(L.ertgb_response_complex(fop_c._ctx, ctypes.c_void_p(zr.data_ptr()),
                                                  ctypes.c_void_p(zi.data_ptr()), ctypes.c_void_p(out_c[0].data_ptr()),
                                                  ctypes.c_void_p(out_c[1].data_ptr()), ctypes.c_void_p(stream)))
            fop_c._check(L.ertgb_jacobian_complex(fop_c._ctx, ctypes.c_void_p(zr.data_ptr()),
                                                  ctypes.c_void_p(zi.data_ptr()), Cc, ctypes.c_void_p(Jc.data_ptr()),
                                                  ctypes.c_void_p(stream)))

        step_c()
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record()
        step_c()
        f1.record()
        torch.cuda.synchronize()
        stc = fop_c.stats()
        res = {"value": f0.elapsed_time(f1) / 1e3, "unit": UNIT, "steps": 1,
               "solver": f"block COCG (Jacobi), {precision} complex, total potential",
               "cocg_iterations": stc["iterations"],
               "columns_finished_fp64": stc["stalled_columns"], "jacobian": "complex FP64"}
        del Jc, fop_c
        torch.cuda.empty_cache()
        return res

    wl_main = (mesh, data, rho)
    plain = fsai_form = cx_form = cem_form = c2_forms = ic0_form = None
    if not args.no_plain and (args.precision, args.precond) != ("fp64", "jacobi"):
        plain = time_form(wl_main, "fp64", "jacobi", 0, "block PCG (Jacobi), FP64",
                          n_steps=max(1, min(args.steps, 2)), n_warm=1, ref_rhoa=rhoa_d)
        plain["ratio_to_value"] = plain["value"] / value
    if not args.no_plain and args.precond != "ic0":
        # the FP64 solver with the incomplete-Cholesky preconditioner
        ic0_form = time_form(wl_main, "fp64", "ic0", 0, "block PCG (IC(0)), FP64",
                             n_steps=max(1, min(args.steps, 2)), n_warm=1, ref_rhoa=rhoa_d)
        ic0_form["ratio_to_value"] = ic0_form["value"] / value
    if not args.no_plain and args.precond == "learned":
        fsai_form = time_form(wl_main, args.precision, "fsai", jdt, f"block PCG (FSAI), {args.precision}",
                              ref_rhoa=rhoa_d)
        fsai_form["ratio_to_value"] = fsai_form["value"] / value
    # the 96-electrode configuration beside the target one, and the variants
    # (complex resistivity, CEM electrodes) on it
    if not args.no_plain or args.cem_only:
        if args.workload == "box_3d":
            wl_c2 = wl_main
        else:
            m2, d2, r2, _ = workload("box_3d")
            wl_c2 = (m2, d2, r2)
    if not args.no_plain and args.workload != "box_3d":
        head = time_form(wl_c2, args.precision, args.precond, jdt, f"block PCG ({args.precond}), {args.precision}",
                         weights_=default_weights("box_3d") if args.precond == "learned" else None)
        ref2 = head.pop("rhoa")
        c2_forms = {"workload": workload_label("box_3d", *wl_c2), "headline_form": head,
                    "plain_fp64_gpu_pcg": time_form(wl_c2, "fp64", "jacobi", 0, "block PCG (Jacobi), FP64",
                                                    ref_rhoa=ref2)}
        if args.precond == "learned":
            c2_forms["fsai_form"] = time_form(wl_c2, args.precision, "fsai", jdt,
                                              f"block PCG (FSAI), {args.precision}", ref_rhoa=ref2)
        c2_forms["ratio_plain_to_headline"] = c2_forms["plain_fp64_gpu_pcg"]["value"] / head["value"]
    c1_forms = None
    if not args.no_plain and args.workload != "line_2d":
        # the 2.5-D configuration (41 electrodes, 17 wavenumbers): the banded
        # direct solve beside the plain FP64 PCG (FP64 Jacobians)
        m1, d1, r1, _ = workload("line_2d")
        wl_c1 = (m1, d1, r1)
        band = time_form(wl_c1, "fp64", "band", 0, "banded Cholesky (direct), FP64")
        ref1 = band.pop("rhoa")
        c1_forms = {"workload": workload_label("line_2d", m1, d1), "band_direct": band,
                    "plain_fp64_gpu_pcg": time_form(wl_c1, "fp64", "jacobi", 0, "block PCG (Jacobi), FP64",
                                                    ref_rhoa=ref1)}
        c1_forms["ratio_plain_to_band"] = c1_forms["plain_fp64_gpu_pcg"]["value"] / band["value"]
    if not args.no_plain:
        cx_form = {"workload": "box_3d", "mixed": time_complex(wl_c2, "mixed"), "fp64": time_complex(wl_c2, "fp64")}
    if (not args.no_plain or args.cem_only) and mesh.dim() == 3:
        cem_form = {"workload": "box_3d"}
        for key, (prec, pc, jd, lab) in {"mixed_fsai": ("mixed", "fsai", 1, "block PCG (FSAI), mixed, total potential"),
                                        "fp64": ("fp64", "jacobi", 0, "block PCG (Jacobi), FP64, total potential")}.items():
            try:
                cem_form[key] = time_cem(wl_c2, prec, pc, jd, lab)
            except Exception as exc:  # the record reports it; the headline line stays
                cem_form[key] = {"error": f"{type(exc).__name__}: {exc}"}

    # roofline of the dominant kernel (CUDA events on the context stream)
    ms = ctypes.c_double()
    by = ctypes.c_double()
    fl = ctypes.c_double()
    prof = {}
    spmm_kind = ("spmm", 0) if args.precision == "fp64" else ("spmm32", 3)
    # the Jacobian is timed in the precision of the step (kernel 1: FP64 J, 4: FP32 J) into its own J buffer
    for name, kid, reps in ((spmm_kind[0], spmm_kind[1], 20), ("jacobian", 1 if jdt == 0 else 4, 3),
                            ("assemble", 2, 10)):
        fop._check(L.ertgb_profile_kernel(fop._ctx, kid, reps, ctypes.c_void_p(J_d.data_ptr()),
                                          ctypes.byref(ms), ctypes.byref(by), ctypes.byref(fl)))
        prof[name] = (ms.value, by.value, fl.value)
    per_step = {spmm_kind[0]: prof[spmm_kind[0]][0] * st["iterations"],
                "jacobian": prof["jacobian"][0],
                "assemble": prof["assemble"][0]}
    dom = max(per_step, key=per_step.get)
    peak, peak_kind = measured_peaks()
    d_ms, d_bytes, d_flops = prof[dom]
    achieved = d_bytes / (d_ms * 1e-3) / 1e9
    traffic = ncu_traffic(f"{dom}{'32' if dom == 'jacobian' and jdt == 1 else ''}_{args.precision}_{args.workload}.txt")
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                "algorithmic_bytes": d_bytes, "ms_per_launch": d_ms,
                "tflops": d_flops / (d_ms * 1e-3) / 1e12,
                "share_of_step": per_step[dom] / (total_ms / args.steps),
                "kernels": {k: {"ms_per_launch": v[0], "algorithmic_bytes": v[1],
                                "gbs": v[1] / (v[0] * 1e-3) / 1e9, "frac": v[1] / (v[0] * 1e-3) / 1e9 / peak}
                            for k, v in prof.items()}}
    del J_d
    torch.cuda.empty_cache()

    # end to end through the reference-facing C ABI with host buffers: the
    # per-cell model copied in for the response and for the Jacobian's
    # scaling, the apparent resistivities and the full Jacobian copied out
    e2e = None
    if not args.no_e2e:
        rho_h = np.ascontiguousarray(rho, np.float64)
        rhoa_h = np.empty(D, np.float64)
        # a plain host array allocated and touched once, as a Gauss-Newton
        # loop reuses it (on the GB300 machine's host the copy into it ran at
        # 40-190 GB/s from run to run; into page-locked or huge-page host
        # buffers it was not faster)
        Jh = np.empty((D, P), dtype=np.float64 if jdt == 0 else np.float32)
        Jh.reshape(-1)[:: 4096 // Jh.itemsize] = 0
        tt, tr, its, tj = [], [], [], []
        for i in range(max(1, min(args.steps, 3)) + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fop._check(L.ertgb_response_host(fop._ctx, rho_h.ctypes.data, rhoa_h.ctypes.data))
            t1 = time.perf_counter()
            fop._check(L.ertgb_jacobian_host(fop._ctx, rho_h.ctypes.data, C, Jh.ctypes.data, jdt))
            if i > 0:
                tt.append(time.perf_counter() - t0)
                tr.append(t1 - t0)
                its.append(fop.stats()["iterations"])
                tj.append(fop.stats()["ms_jacobian"] * 1e-3)
        jbytes = D * P * Jh.itemsize
        copy_s = float(np.mean(tt) - np.mean(tr) - np.mean(tj))
        e2e = {"value": float(np.mean(tt)), "unit": UNIT, "h2d_bytes_per_step": int(2 * C * 8),
               "d2h_bytes_per_step": int(D * 8 + jbytes), "steps": len(tt),
               "path": "ertgb_response_host + ertgb_jacobian_host (host numpy buffers, allocated once)",
               "response_s": float(np.mean(tr)), "jacobian_with_copy_s": float(np.mean(tt) - np.mean(tr)),
               "jacobian_copy_gbs": jbytes / copy_s / 1e9 if copy_s > 0 else None,
               "pcg_iterations": its,
               "check_rhoa_vs_device": float(np.max(np.abs(rhoa_h - rhoa_d.cpu().numpy()) / rhoa_h))}
        del Jh

    gn = None
    if args.gn and rank == 0:
        gn = gn_iteration(args, mesh, data, rho, local, weights)

    refine_rec = None
    if rank == 0 and not args.no_plain:
        # the forward-mesh refinement pyGIMLi applies to a parameter mesh
        # (H2): device (ertgb_refine, incl. transfers) vs the host restatement
        from pygimli_gb300 import refine as _refine
        _refine.createH2(mesh, local)
        t0 = time.perf_counter()
        mh = _refine.createH2(mesh, local)
        t_dev = time.perf_counter() - t0
        t0 = time.perf_counter()
        mesh.createH2()
        t_host = time.perf_counter() - t0
        refine_rec = {"what": "H2 of the workload mesh", "cells_in": mesh.cellCount(), "cells_out": mh.cellCount(),
                      "nodes_out": mh.nodeCount(), "device_s": t_dev, "host_numpy_s": t_host}
        del mh

    cpu = None
    if cpu_p is not None:
        try:
            r = cpu_q.get(timeout=600)
        except Exception as exc:  # queue.Empty: the baseline did not finish in time
            r = {"error": f"CPU baseline did not finish: {type(exc).__name__}"}
        cpu_p.join(timeout=5)
        if "error" in r:
            cpu = {"value": None, "unit": UNIT, "cores": 1, "kind": "port", "sample": r["error"]}
        else:
            cpu = {"value": r["value"], "unit": UNIT, "cores": 1, "kind": "port",
                   "sample": r["desc"] + f"; sample wall {r['wall_s']:.1f} s (ran beside the GPU timings)"}

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": value * 1e3 * world, "higher_is_better": False,
               "scaling": "weak", "vs_baseline": None,
               "dtype": "f64" if args.precision == "fp64" else "f32+f64 (FP32 PCG, FP64 reliable updates)",
               "data": "synthetic (seeded)",
               "config": dict(cfg, parallelism=f"replicas x{world}",
                              solver=f"block PCG ({args.precond}), {args.precision}",
                              jacobian="FP64" if jdt == 0 else "FP32 (FP64 differences)",
                              rtol=args.rtol, l2="working set > L2: PCG blocks 4 x "
                              f"{mesh.nodeCount() * fop.sizes()[3] * 8 / 1e6:.0f} MB, J "
                              f"{D * P * (8 if jdt == 0 else 4) / 1e9:.1f} GB"),
               "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
               "plain_fp64_gpu_pcg": plain, "fsai_form": fsai_form, "fp64_ic0_form": ic0_form,
               "box_3d_forms": c2_forms, "line_2d_forms": c1_forms,
               "gn_iteration": gn, "refine_h2": refine_rec, "complex_form": cx_form, "cem_form": cem_form,
               "learned_weights": os.path.relpath(weights, ROOT) if weights else None,
               "clocks": clk, "step_ms": step_ms,
               "breakdown_ms": {"assemble": st["ms_assemble"], "rhs": st["ms_rhs"], "solve": st["ms_solve"],
                                "collect": st["ms_collect"], "jacobian": st["ms_jacobian"],
                                "pcg_iterations": st["iterations"], "n_rhs": st["n_rhs"],
                                "max_rel_residual": st["max_rel_residual"],
                                "stalled_columns_fp64_finish": st["stalled_columns"], "setup_s": setup_s}}
        print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.case:
        run_case(args)
        return
    world, rank, local = dist_init(args.gpus if args.impl == "ours" else 0)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
