"""Trains the learned ICP warm start on the GPU and evaluates it against
plain ICP.

    python -m merge_fusion_gb300.train_proposer --out weights.npz

Data: seeded synthetic room trajectories (the benchmark's scene generator,
640x480 uint16 depth); pairs (a, a+k), k in {1, 2, 3}; labels from plain ICP
run to convergence.  Training: Adam on the standardised labels with a cosine
learning-rate schedule, batch 256, on the library's own BF16 tensor-core
forward and backward kernels.  Evaluation: held-out trajectories (disjoint
seeds); ICP iterations to converge (RMS change < 1e-4 m), learned vs plain,
the final pose difference and the fallbacks.  Prints one JSON line."""
import argparse
import json
import time

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    # the defaults give 500 x (134 - 3) x 3 = 196,500 training pairs and 8
    # held-out trajectories for the 1000 evaluation pairs
    ap.add_argument("--train-trajectories", type=int, default=500)
    ap.add_argument("--eval-trajectories", type=int, default=8)
    ap.add_argument("--frames", type=int, default=134)
    ap.add_argument("--steps", type=int, default=8000)
    ap.add_argument("--eval-pairs", type=int, default=1000)
    ap.add_argument("--seed", type=int, default=1000)
    ap.add_argument("--eval-only", help="evaluate saved weights instead of training")
    args = ap.parse_args()
    import torch
    from . import proposer as mp
    torch.cuda.set_device(0)
    net = mp.PoseProposer(max_batch=256)
    if args.eval_only:
        params, mean, std = mp.load(args.eval_only)
        net.set_params(params)
        eval_seeds = list(range(args.seed + 10000, args.seed + 10000 + args.eval_trajectories))
        res = mp.evaluate(net, mean, std, eval_seeds, args.frames, max_pairs=args.eval_pairs)
        print(json.dumps(res), flush=True)
        return
    net.set_params(mp.init_params(args.seed))
    t0 = time.perf_counter()
    train_seeds = list(range(args.seed, args.seed + args.train_trajectories))
    x, y, _ = mp.make_pairs(net, train_seeds, args.frames)
    t1 = time.perf_counter()
    mean, std, hist = mp.train(net, x, y, steps=args.steps, seed=args.seed)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    eval_seeds = list(range(args.seed + 10000, args.seed + 10000 + args.eval_trajectories))
    res = mp.evaluate(net, mean, std, eval_seeds, args.frames, max_pairs=args.eval_pairs)
    t3 = time.perf_counter()
    params = net.get_params()
    info = {"train_pairs": int(x.shape[0]), "train_trajectories": args.train_trajectories,
            "frames_per_trajectory": args.frames, "steps": args.steps, "loss_first": hist[0][1],
            "loss_last": hist[-1][1], "seed": args.seed}
    mp.save(args.out, params, mean, std, info)
    line = dict(info)
    line.update(res)
    line.update({"seconds_data": round(t1 - t0, 1), "seconds_train": round(t2 - t1, 1),
                 "seconds_eval": round(t3 - t2, 1), "loss_history": hist})
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
