"""Train the learned preconditioner on the GPU for a workload and save its
weights (the packaged ones under pygimli_gb300/weights/ come from this):

    python -m pygimli_gb300.train_learned --workload box_3d --steps 1500 \\
        --out pygimli_gb300/weights/box_3d.npz

Training models: seeded log-normal backgrounds with blocky inclusions of
1e2-1e5 contrast (``synthetic.random_models``) on the workload's mesh; the
system matrices come from the library's own FP64 assembly.  Held-out models
then measure what the network gains: Kaporin's number and the PCG
iterations / solve time of the mixed-precision solver with Jacobi, with the
network, and with FSAI (the minimiser of the training loss on this pattern).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def meshes_for(workload):
    from . import synthetic
    if workload == "box_3d":
        mesh, data, _ = synthetic.box_3d(scheme="inline")
        return [(mesh, data)]
    if workload == "box_3d_p2":
        mesh, data, _ = synthetic.box_3d(scheme="inline")
        return [(mesh.createP2(), data)]
    if workload == "line_2d":
        mesh, data, _ = synthetic.line_2d()
        return [(mesh, data)]
    raise ValueError(workload)


def evaluate(fop, lp, models):
    """Per preconditioner: total PCG iterations, solve ms and the max relative
    apparent-resistivity difference to the Jacobi solve."""
    out = {}
    ref = {}
    for name in ("jacobi", "learned", "fsai"):
        fop.setPreconditioner(name, lp if name == "learned" else None)
        its, ms, dev = 0, 0.0, 0.0
        for i, m in enumerate(models):
            r = fop.response(m)
            st = fop.stats()
            its += st["iterations"]
            ms += st["ms_solve"]
            if name == "jacobi":
                ref[i] = r
            else:
                dev = max(dev, float(np.max(np.abs(r - ref[i]) / ref[i])))
        out[name] = {"iterations": its, "ms_solve": ms, "max_rel_diff_rhoa_vs_jacobi": dev}
    fop.setPreconditioner("jacobi")
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="box_3d", choices=["box_3d", "box_3d_p2", "line_2d"])
    ap.add_argument("--models", type=int, default=48)
    ap.add_argument("--held-out", type=int, default=4)
    ap.add_argument("--steps", type=int, default=1500)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--lr-final", type=float, default=2e-4)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", required=True)
    a = ap.parse_args(argv)
    from . import ERTModelling, synthetic
    from .learned import LearnedPreconditioner
    tasks, held = [], []
    for mi, (mesh, data) in enumerate(meshes_for(a.workload)):
        fop = ERTModelling(precision="mixed")
        fop.setData(data)
        fop.setMesh(mesh, ignoreRegionManager=True)
        models = synthetic.random_models(mesh, a.models + a.held_out, seed=1000 * (a.seed + 1) + mi)
        tasks.append((fop, models[:a.models]))
        held.append((fop, models[a.models:]))
    lp = LearnedPreconditioner(seed=a.seed)
    k_before = float(np.mean([lp.loss(f, m) for f, ms in held for m in ms]))
    t0 = time.time()
    hist = lp.train(None, None, a.steps, lr=a.lr, lr_final=a.lr_final, tasks=tasks, log_every=max(1, a.steps // 10))
    train_s = time.time() - t0
    k_after = float(np.mean([lp.loss(f, m) for f, ms in held for m in ms]))
    ev = {}
    for i, (fop, ms) in enumerate(held):
        ev[f"mesh{i}"] = evaluate(fop, lp, ms)
    meta = {"workload": a.workload, "steps": a.steps, "models": a.models, "held_out": a.held_out,
            "train_s": train_s, "kaporin_held_out_before": k_before, "kaporin_held_out_after": k_after,
            "eval": ev}
    print(json.dumps(meta), flush=True)
    lp.save(a.out, meta=json.dumps(meta), history=np.array(hist))


if __name__ == "__main__":
    main()
