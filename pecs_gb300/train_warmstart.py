"""Train the learned warm start on the GPU and report what it gains.

    python -m pecs_gb300.train_warmstart --n-train 4096 --n-eval 512 --out model.npz

1. Draws n_train + n_eval parameter sets (seeded) from the benchmark's
   distributions (pecs_gb300.learned.RANGES).
2. Marches every training draw to steady state with the plain method
   (streamed through 64 slots, ``--precision``).
3. Builds the POD basis of [log n | log p | Phi] and trains the MLP with the
   library's BF16/FP32 kernels (Adam, cosine decay).
4. On the held-out draws: prediction error, steps to steady state with and
   without the warm start, fallback rate, interface currents of both runs.
Writes the model (MLP parameters + POD basis) and a JSON report.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-train", type=int, default=4096)
    ap.add_argument("--n-eval", type=int, default=512)
    ap.add_argument("--refine", type=int, default=6)
    ap.add_argument("--rank", type=int, default=64)
    ap.add_argument("--hidden", type=int, default=512)
    ap.add_argument("--epochs", type=int, default=600)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--out", default="warmstart.npz")
    ap.add_argument("--report", default="warmstart_report.json")
    args = ap.parse_args()

    import torch

    import pecs_gb300 as pg
    from pecs_gb300 import learned as L

    pg.build()
    prec = pg.PREC_FP32_MIXED if args.precision == "mixed" else pg.PREC_FP64
    base = pg.half_cell(n_refine=args.refine)
    B = 64
    thetas = L.sample(args.n_train + args.n_eval, args.seed)
    tr, ev = thetas[:args.n_train], thetas[args.n_train:]
    ctx = pg.Context([L.instance_params(t, base) for t in tr[:B]], precision=prec)
    lay = L.Layout.of(ctx)
    t0 = time.perf_counter()
    Y, steps_tr = L.steady_states(ctx, tr, base)
    t_gen = time.perf_counter() - t0
    print(f"generated {len(tr)} steady states in {t_gen:.1f}s, median steps {np.median(steps_tr):.0f}")
    op = L.NeuralOperator(rank=args.rank, hidden=args.hidden, seed=args.seed)
    T = op.fit_basis(Y, lay)
    X = torch.from_numpy(L.normalize(tr)).cuda()
    t0 = time.perf_counter()
    hist = op.train(X, T, epochs=args.epochs, batch=args.batch, lr=args.lr, seed=args.seed, log=print)
    t_train = time.perf_counter() - t0
    # held-out evaluation
    Yev, steps_plain = L.steady_states(ctx, ev, base)
    Xev = torch.from_numpy(L.normalize(ev)).cuda()
    P = op.predict(Xev)
    err = {}
    names = ("log_n", "log_p", "Phi")
    blocks = ((0, lay.n_u), (lay.n_u, 2 * lay.n_u), (2 * lay.n_u, lay.n_out))
    for nm, (a, b) in zip(names, blocks):
        d = (P[:, a:b] - Yev[:, a:b]).norm(dim=1) / Yev[:, a:b].norm(dim=1).clamp_min(1e-30)
        err[nm] = {"median": float(d.median()), "max": float(d.max())}
    # held-out sweeps, streamed: warm-started and from the standard initial condition
    steps_warm, fallbacks, cur_warm, _ = L.stream_warm_sweep(ctx, op, ev, base)
    steps_std, _, cur_plain, _ = L.stream_warm_sweep(ctx, None, ev, base)
    steps_warm = np.asarray(steps_warm)
    m = len(steps_warm)
    cur_warm, cur_plain = np.asarray(cur_warm), np.asarray(cur_plain)
    rep = {
        "n_train": args.n_train, "n_eval": args.n_eval, "refine": args.refine, "rank": args.rank,
        "hidden": args.hidden, "n_params": op.mlp.n_params, "epochs": args.epochs,
        "precision": args.precision, "seed": args.seed,
        "gen_seconds": t_gen, "train_seconds": t_train,
        "final_loss": float(hist[-1]) if hist else None, "first_loss": float(hist[0]) if hist else None,
        "prediction_rel_error": err,
        "steps_plain_median": float(np.median(steps_plain[:m])),
        "steps_plain_streamed_median": float(np.median(steps_std)),
        "steps_warm_median": float(np.median(steps_warm)),
        "steps_saved_fraction": float(1.0 - steps_warm.sum() / steps_plain[:m].sum()),
        "fallback_rate": float(np.mean(fallbacks)),
        "current_rel_diff_max": float(np.max(np.abs(cur_warm - cur_plain) /
                                             np.maximum(np.abs(cur_plain), 1e-30))),
        "pod_singular_values_head": [float(v) for v in op.sv[:8].tolist()],
    }
    print(json.dumps(rep, indent=1))
    np.savez_compressed(args.out, params=op.mlp.get_params(), widths=np.array(op.mlp.widths),
                        mean=op.mean.cpu().numpy(), scale=op.scale.cpu().numpy(),
                        basis=op.basis.float().cpu().numpy(), cscale=op.cscale.cpu().numpy(),
                        refine=args.refine, rank=args.rank)
    with open(args.report, "w") as fh:
        json.dump(rep, fh, indent=1)


if __name__ == "__main__":
    main()
