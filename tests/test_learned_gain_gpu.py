"""What the trained network gains.  The shipped weights
(nekbench_gb300/weights/precond_n7_c16.bin: N=7, 16 channels, trained by the
library's own forward/backward kernels on 200 seeded problems) against plain
Jacobi on held-out problems of the training workload: N=7, E=24^3 perturbed
box, lambda1 = 1 + 0.5 sin(2 pi k.x) with k drawn from the seed, both solvers
to a true FP64 relative residual of 1e-8 (mixed FP32 Krylov iteration with
FP64 residual replacement; the learned one as flexible CG with five kept
directions).  Seeds 1000-1002 were never seen in training (training used
0-199).  The network must cut the iteration count on every seed, by at least
15 % (the 50-seed evaluation of these weights measured 23 %); both solves must
converge.  The iterations and times are printed for the record."""
import os

import pytest

pytestmark = pytest.mark.gpu

WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                       "nekbench_gb300", "weights", "precond_n7_c16.bin")


def test_trained_network_cuts_iterations_on_held_out_problems(nb, dev):
    import torch

    from nekbench_gb300 import learned as LP
    net = nb.Net.load(WEIGHTS)
    assert net.inference == nb.NET_TENSOR
    bp = nb.BP(7, 24, 24, 24, perturb=0.1, seed=3)
    ev = LP.evaluate(bp, net, range(1000, 1003), torch, dev)
    for row in ev["rows"]:
        j, l = row["jacobi"], row["learned"]
        print(f"seed {row['seed']}: Jacobi {j['iterations']} it {j['elapsed_s']:.3f} s, "
              f"learned {l['iterations']} it {l['elapsed_s']:.3f} s")
        assert j["status"] == 0 and l["status"] == 0
        assert j["true_rel_res"] <= 1e-8 and l["true_rel_res"] <= 1e-8
        assert l["iterations"] * 1.15 <= j["iterations"], row
    assert ev["all_converged"] and ev["iteration_ratio"] >= 1.15
