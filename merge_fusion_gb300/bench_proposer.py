"""Times the learned pose proposer at batch 256 on the GPU.

    python -m merge_fusion_gb300.bench_proposer [n]

Three warm-up rounds, then n forward passes and n training steps (forward,
backward, Adam), each a synchronous library call timed on the host."""
import sys
import time

import numpy as np


def main():
    import torch
    from . import proposer as mp
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 50
    net = mp.PoseProposer(max_batch=256)
    net.set_params(mp.init_params(0))
    rng = np.random.default_rng(0)
    x = torch.from_numpy(rng.uniform(0.4, 4, (256, 60, 80, 2)).astype(np.float16)).cuda()
    t = torch.from_numpy(rng.normal(size=(256, 6)).astype(np.float32)).cuda()
    for _ in range(3):
        net.train_step(x, t, 1e-4)
        net.predict(x)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(n):
        net.predict(x)
    t1 = time.perf_counter()
    for _ in range(n):
        net.train_step(x, t, 1e-4)
    t2 = time.perf_counter()
    print("batch 256: forward %.3f ms, train step %.3f ms" % ((t1 - t0) / n * 1e3, (t2 - t1) / n * 1e3))


if __name__ == "__main__":
    main()
