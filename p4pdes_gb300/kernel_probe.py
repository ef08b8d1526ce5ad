"""Times one finest-level kernel of a solver on resident data (the library's
fishgpu_solver_time_kernel), after one solve that fills the vectors:

    python -m p4pdes_gb300.kernel_probe --opts "-fsh_dim 3 -da_refine 8 ..." --kernel cgp_apply_acc --reps 20

Prints the mean ms per launch, the algorithmic bytes and GB/s.  Profilers
can capture the timed launches (one kernel, a few launches)."""
import argparse

import torch

import p4pdes_gb300 as fg


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--opts", required=True, help="fish options, as for the fish driver")
    ap.add_argument("--kernel", required=True, help="a name fishgpu_solver_time_kernel accepts")
    ap.add_argument("--reps", type=int, default=20)
    a = ap.parse_args(argv)
    o = fg.options(a.opts)
    with fg.Solver(o) as s:
        u = torch.empty(o.shape, dtype=torch.float64, device="cuda")
        s.solve(u)
        ms, by = s.time_kernel(a.kernel, a.reps)
    print("%s: %.4f ms per launch, %.3e algorithmic bytes, %.0f GB/s" % (a.kernel, ms, by, by / ms / 1e6 if ms else 0))


if __name__ == "__main__":
    main()
