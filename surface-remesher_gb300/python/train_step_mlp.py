"""Train the learned-step MLP on plain Lloyd trajectories and evaluate it.

    python train_step_mlp.py train [--runs 200] [--horizon 8] [--sites 4096,8192,16384] [--out DIR]
    python train_step_mlp.py eval [--config plain_4096] [--params FILE]

train: plain Lloyd runs on the config-0 density family (1024^2 grids, 8
seeded Gaussians in the disk, seeds 1000 + run) with 4096, 8192 or 16384
uniform sites in turn (mean cell radii of 7.6, 5.4 and 3.8 pixels) and site
ids tracked; every 2 iterations up to 40 the features of every site are
recorded (about 2048 sites per record), and each site's target is its
displacement over the next `horizon` iterations (or to where it is after 200
iterations), in units of the mean cell radius (sites merged on the way are
dropped).  The MLP is
trained on the GPU (gcvt_mlp_train) and its parameters are written to
DIR/step_mlp.npy with DIR/step_mlp.json describing the run; the defaults
made the parameters in surface-remesher_gb300/data.

eval: time to reach E <= (1 + 1e-4) E_conv, E_conv the energy after 1000
plain iterations, for plain Lloyd and for Lloyd with gated learned steps,
on one configuration (the device stops each run at the target); prints one
JSON line.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import gcvt_gb300 as G  # noqa: E402
from workloads import CONFIGS, config_inputs, disk_sites, gaussian_density  # noqa: E402

DATA = os.path.normpath(os.path.join(HERE, "..", "data"))
N, K, A_MAX, S_LO, S_HI, SITES = 1024, 8, 4.0, 0.02, 0.15, 4096
RECORD = list(range(2, 41, 2))
T_FINAL = 200


def mean_radius(rho, sites):
    """The features' unit as the library computes it: sqrt(support pixels /
    sites / pi), support = per-row [first, last] span of nonzero density."""
    nz = rho != 0
    rows = nz.any(1)
    first = np.argmax(nz, 1)
    last = rho.shape[1] - 1 - np.argmax(nz[:, ::-1], 1)
    px = int(((last - first + 1) * rows).sum())
    return max(np.sqrt(px / max(sites, 1) / np.pi), 0.5)


def collect(runs, horizon, keep=0.5, seed=0, site_counts=(SITES,)):
    """Samples (features, target) of plain runs: the target of a site seen at
    iteration t is its displacement to iteration t + horizon (horizon 0: to
    iteration T_FINAL), in mean cell radii.  Run r has site_counts[r % k]
    sites (more sites: smaller cells, in pixels); every run keeps about
    keep * 4096 sites per recorded iteration."""
    rng = np.random.default_rng(seed)
    ctx = G.Context(N)
    ctx.learning(True, track_ids=True)
    out = []
    last = T_FINAL if horizon <= 0 else RECORD[-1] + horizon
    for r in range(runs):
        m = int(site_counts[r % len(site_counts)])
        rho = gaussian_density(N, K, A_MAX, S_LO, S_HI, 1000 + r)
        sites = disk_sites(N, m, 1000 + r, rho)
        ctx.load(sites, rho, np.zeros((N, N), np.uint8))
        rbar = mean_radius(rho, m)
        frac = keep * min(1.0, SITES / m)
        snaps, pos = {}, {}
        for t in range(1, last + 1):
            ctx.iterate(1)
            if t in RECORD or (horizon > 0 and t - horizon in RECORD) or t == last:
                f, ids, xy = ctx.features(with_ids=True)
                p = np.full((m, 2), np.nan, np.float32)
                p[ids] = xy
                pos[t] = p
                if t in RECORD:
                    snaps[t] = (f, ids, xy)
        for t, (f, ids, xy) in snaps.items():
            end = pos[last] if horizon <= 0 else pos[t + horizon]
            tgt = (end[ids] - xy) / rbar
            ok = np.isfinite(tgt).all(1) & (rng.random(len(ids)) < frac)
            out.append(np.concatenate([f[ok], tgt[ok]], 1).astype(np.float32))
    ctx.close()
    return np.concatenate(out)


def train(args):
    t0 = time.time()
    counts = tuple(int(v) for v in str(args.sites).split(","))
    samples = collect(args.runs, args.horizon, site_counts=counts)
    t1 = time.time()
    p0 = G.mlp_init(args.seed)
    params, loss = G.mlp_train(samples, p0, steps=args.steps, batch=args.batch, lr=args.lr,
                               seed=args.seed)
    t2 = time.time()
    os.makedirs(args.out, exist_ok=True)
    np.save(os.path.join(args.out, "step_mlp.npy"), params.astype(np.float32))
    meta = {"runs": args.runs, "samples": int(len(samples)), "steps": args.steps,
            "batch": args.batch, "lr": args.lr, "seed": args.seed,
            "grid": N, "sites": list(counts), "gaussians": K, "record": RECORD,
            "horizon": args.horizon if args.horizon > 0 else T_FINAL,
            "loss_first": float(loss[:20].mean()), "loss_last": float(loss[-50:].mean()),
            "target_var": float(samples[:, 10:].var(0).sum() / 2),
            "collect_s": t1 - t0, "train_s": t2 - t1}
    with open(os.path.join(args.out, "step_mlp.json"), "w") as fh:
        json.dump(meta, fh, indent=1)
    print(json.dumps(meta))


def time_to_energy(ctx, sites, rho, mask, target, learned, jump_every, limit):
    """(seconds, iterations, jumps tried, jumps kept) until the first
    iteration whose energy is at most target: the device stops the run there
    (gcvt_ctx_set_target_energy), timed with CUDA events on the context's
    stream around the whole run after the load."""
    import torch
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.set_target_energy(target)
    ctx.load(sites, rho, mask)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    tried = kept = 0
    if learned:
        tried, kept = ctx.iterate_learned(limit, jump_every)
    else:
        ctx.iterate(limit)
    e1.record(stream)
    e1.synchronize()
    it = ctx.info()["iterations"]
    ctx.set_target_energy(0)
    ctx.set_stream(None)
    return e0.elapsed_time(e1) / 1e3, it, tried, kept


def evaluate(args):
    sites, rho, mask, _ = config_inputs(args.config, seed=1)
    n = sites.shape[0]
    ctx = G.Context(n)
    ctx.load(sites, rho, mask)
    ctx.iterate(args.conv_iters)
    e_conv = ctx.info()["energy"]
    target = e_conv * (1 + 1e-4)
    plain = time_to_energy(ctx, sites, rho, mask, target, False, 0, args.conv_iters)
    params = np.load(args.params)
    lctx = G.Context(n)
    lctx.learning(True)
    lctx.set_mlp(params)
    learned = time_to_energy(lctx, sites, rho, mask, target, True, args.jump_every,
                             args.conv_iters)
    line = {"config": args.config, "e_conv": e_conv, "target": target,
            "conv_iters": args.conv_iters,
            "plain": {"s": plain[0], "iterations": plain[1]},
            "learned": {"s": learned[0], "iterations": learned[1], "jumps_tried": learned[2],
                        "jumps_kept": learned[3], "jump_every": args.jump_every},
            "speedup": plain[0] / learned[0]}
    print(json.dumps(line))
    ctx.close()
    lctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("mode", choices=["train", "eval"])
    ap.add_argument("--runs", type=int, default=200)
    ap.add_argument("--steps", type=int, default=8000)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=DATA)
    ap.add_argument("--config", default="plain_4096", choices=sorted(CONFIGS))
    ap.add_argument("--params", default=os.path.join(DATA, "step_mlp.npy"))
    ap.add_argument("--conv-iters", type=int, default=1000)
    ap.add_argument("--jump-every", type=int, default=4)  # three plain iterations, one learned step
    ap.add_argument("--sites", default="4096,8192,16384",
                    help="site counts of the training runs, comma-separated, used in turn")
    ap.add_argument("--horizon", type=int, default=8,
                    help="target: displacement over this many iterations (0: to iteration 200)")
    args = ap.parse_args()
    if args.mode == "train":
        train(args)
    else:
        evaluate(args)


if __name__ == "__main__":
    main()
