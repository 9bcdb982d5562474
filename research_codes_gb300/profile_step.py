"""One steady-state force evaluation bracketed for a profiler.

    python -m research_codes_gb300.profile_step --config c2 --scale 0.3 [--precision fp32c]

Builds the configuration's particle system, evaluates the forces until the
smoothing lengths have converged (one density walk), then runs one more
evaluation between cudaProfilerStart and cudaProfilerStop, so that
`ncu --profile-from-start off` captures exactly the kernels of a steady
force evaluation.  Prints the phase times (CUDA events) of that evaluation.
With --what step the settling and the profiled call are whole steps
(kick-drift, forces with search-radius re-walks, correction).
"""
import argparse
import ctypes
import json

from . import functors, ic
from .system import ParticleSystem, state_from_ic


def _driver_profiler():
    """cuProfilerStart / cuProfilerStop of the CUDA driver (the runtime the
    library links statically and torch's runtime share the driver)."""
    drv = ctypes.CDLL("libcuda.so.1")
    return drv.cuProfilerStart, drv.cuProfilerStop


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2")
    ap.add_argument("--scale", type=float, default=0.3)
    ap.add_argument("--precision", default="fp32c")
    ap.add_argument("--n-group", type=int, default=256)
    ap.add_argument("--quadrupole", type=int, default=0, help="1: quadrupole tree gravity")
    ap.add_argument("--item-split-nj", type=int, default=4096)
    ap.add_argument("--heavy-classes", type=int, default=2)
    ap.add_argument("--gravity-jtile", type=int, default=32)
    ap.add_argument("--settle", type=int, default=4, help="force evaluations before the profiled one")
    ap.add_argument("--what", choices=("forces", "step"), default="forces",
                    help="profile one force evaluation or one whole step (after --settle steps)")
    args = ap.parse_args()
    import torch
    torch.cuda.init()
    s, eta = ic.config_system(args.config, scale=args.scale)
    s = state_from_ic(s)
    n = len(s["mass"])
    with functors.Context(precision=args.precision, eta=eta) as ctx:
        ps = ParticleSystem(ctx, n, n_group=args.n_group, use_graph=0, quadrupole=args.quadrupole,
                            item_split_nj=args.item_split_nj, heavy_classes=args.heavy_classes,
                            gravity_jtile=args.gravity_jtile)
        ps.upload(s)
        for _ in range(args.settle):
            if args.what == "step":
                ps.step(1)
            else:
                ps.compute_forces()        # h converges in place
        start, stop = _driver_profiler()
        torch.cuda.synchronize()
        start()
        if args.what == "step":
            ps.step(1)
        else:
            ps.compute_forces()
        torch.cuda.synchronize()
        stop()
        out = {"n": n, "stats": ps.stats(), "phases_ms": ps.phase_times()}
        print(json.dumps(out))
        ps.close()


if __name__ == "__main__":
    main()
