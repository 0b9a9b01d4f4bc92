"""Profiling case: a short RGF run on a seeded chain device, sized for kernel profilers.

Not a test (pytest does not collect it): the ncu summaries of the split-product
and inverse kernels are captured on this case.

The batched sweep launches every block product over all points of a wave.
Each launch therefore carries the full per-launch work of a large run: P
points x one n x n complex product. The memory held stays a few GB because
the device has few slabs. Example, 512 points of 128-orbital blocks over 3
slabs (about 3.5 GB on the device):

    python tests/profile_case.py --points 512 --slabs 3

Prints one JSON line with the wall time of each repeat and the number of
points with a non-zero status.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--points", type=int, default=512, help="(E, k) points, a multiple of --nk")
    ap.add_argument("--slabs", type=int, default=3)
    ap.add_argument("--orbitals", type=int, default=128)
    ap.add_argument("--nk", type=int, default=16)
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed", "mixed-fp64"])
    ap.add_argument("--repeat", type=int, default=2)
    a = ap.parse_args(argv)
    if a.points % a.nk:
        ap.error("--points must be a multiple of --nk")

    import torch

    from quantum_transport_gb300 import rgf
    from quantum_transport_gb300.build import build
    from quantum_transport_gb300.devices import make_chain_device

    build()
    nE = a.points // a.nk
    dev = make_chain_device(a.slabs, a.orbitals, nE, -2.0, 2.0, seed=2024, nk=a.nk)
    ctx = rgf.Context(0)
    cm = lambda x: torch.from_numpy(rgf.colmajor(x)).cuda()
    H00, H10 = cm(dev.H00), cm(dev.H10)
    E = torch.from_numpy(dev.E).cuda()
    P, nm = a.points, a.orbitals
    out = {"T": torch.zeros(P, dtype=torch.float64, device="cuda"),
           "tr": torch.zeros(P, dtype=torch.float64, device="cuda"),
           "tre": torch.zeros(P, dtype=torch.float64, device="cuda"),
           "diag_gr": torch.zeros(P * a.slabs * nm, dtype=torch.complex128, device="cuda"),
           "status": torch.zeros(P, dtype=torch.int32, device="cuda")}
    times = []
    for _ in range(a.repeat):
        t0 = time.perf_counter()
        rgf.rgf_solve_device(ctx, H00, nm * nm, 0, H10, 0, 0, nm, a.slabs, a.nk, E, nE, out,
                             precision=a.precision, mul=0.1, mur=-0.1, sancho_tol=1e-10)
        ctx.sync()
        times.append(time.perf_counter() - t0)
    bad = int((out["status"] != 0).sum().item())
    ctx.close()
    print(json.dumps({"points": P, "slabs": a.slabs, "orbitals": nm, "precision": a.precision,
                      "seconds": times, "points_bad_status": bad}))


if __name__ == "__main__":
    main()
