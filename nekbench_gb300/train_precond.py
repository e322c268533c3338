"""Trains the learned element preconditioner on the GPU and evaluates it.

Workload: N=7, E=24^3=13824 box (perturbed trilinear elements, Dirichlet),
training pairs from 200 seeded Jacobi-PCG solves with smooth random
coefficients, 3 layers of 3x3x3 convolutions with 16 channels, GELU, BF16
weights / FP32 accumulation; evaluated on 50 held-out seeds.

  python -m nekbench_gb300.train_precond --out weights/precond_n7_c16.bin --report r.json
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--n", type=int, default=24)
    p.add_argument("--train-seeds", type=int, default=200)
    p.add_argument("--eval-seeds", type=int, default=50)
    p.add_argument("--steps", type=int, default=12000)
    p.add_argument("--batch", type=int, default=4096)
    p.add_argument("--lr", type=float, default=2e-3)
    p.add_argument("--channels", type=int, default=16)
    p.add_argument("--frac", type=float, default=0.125)
    p.add_argument("--target", choices=("local", "pcg"), default="local",
                   help="local: element-interior block solve of the residual; "
                        "pcg: the Jacobi-PCG's own correction over --horizon iterations")
    p.add_argument("--horizon", type=int, default=8,
                   help="target pcg: correction = x_{k+horizon} - x_k (0: x* - x_k)")
    p.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                 "weights", "precond_n7_c16.bin"))
    p.add_argument("--report", default=None)
    a = p.parse_args(argv)

    import torch

    import nekbench_gb300 as nb
    from nekbench_gb300 import learned as LP

    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)

    def log(msg):
        print(msg, flush=True)

    t0 = time.perf_counter()
    bp = nb.BP(7, a.n, a.n, a.n, perturb=0.1, seed=3)
    net = nb.Net(8, a.channels, 3, seed=1)
    inp, tgt = LP.generate_pairs(bp, range(a.train_seeds), torch, dev, frac=a.frac,
                                 horizon=a.horizon, log=log, target=a.target)
    losses = LP.train(net, inp, tgt, torch, steps=a.steps, batch=a.batch, lr=a.lr, log=log)
    del inp, tgt
    torch.cuda.empty_cache()
    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    net.save(a.out)
    ev = LP.evaluate(bp, net, range(1000, 1000 + a.eval_seeds), torch, dev)
    report = {"workload": f"N=7, E={a.n}^3={bp.E}, lambda1 = 1 + 0.5 sin(2 pi k.x), k~U{{1..4}}^3",
              "target": a.target, "horizon": a.horizon,
              "train_seeds": a.train_seeds, "eval_seeds": a.eval_seeds, "steps": a.steps,
              "batch": a.batch, "lr": a.lr, "channels": a.channels,
              "loss_first": losses[0], "loss_last": losses[-1],
              "loss_curve": losses[:: max(1, len(losses) // 20)],
              "evaluation": {k: v for k, v in ev.items() if k != "rows"},
              "rows": ev["rows"], "seconds": time.perf_counter() - t0}
    log(json.dumps(report["evaluation"]))
    if a.report:
        with open(a.report, "w") as fh:
            json.dump(report, fh, indent=1)
    return report


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    main()
