"""Benchmark: batched RGF E-points/s on one GB300 (split-precision tensor-core path).

Workload (the batched configuration): a seeded synthetic device of 100 slabs x
128 orbitals with transverse dispersion over 16 k-points and 4096 energies on
[-2, 2] eV -- 65,536 independent (E, k) solves.  One STEP solves one batch of
``--batch-energies`` energies x 16 k through the whole hot path (both
Sancho-Rubio leads, forward and backward sweeps, Caroli T(E), tr/tre, LDOS
and G^< diagonals); successive steps walk through the 4096-energy grid.

Reported (one JSON line on rank 0):
  value        E-points/s with inputs resident in HBM (device-pointer call)
  e2e          the same through the host-pointer C-ABI call (H blocks and the
               energy slice copied in, all outputs copied out, inside the timer)
  roofline     the dominant kernel (complex64 split product) timed live with
               CUDA events on the library's stream
  cpu_baseline the C restatement of the sweep timed on the host cores
  fp64         the plain-FP64 GPU path on a small sample of the same points
               and the T(E) error of the split path against it

``--impl reference`` times the CPU restatement (the reference's Fortran
cannot be built here: no Fortran compiler is installed).

``--workload uneven`` measures the uneven-block configuration instead: a
4000-atom random tight-binding graph sliced into 25 slabs of 134-184 orbitals,
2048 energies x 8 k-points, every block above one 128-row tile of the split
product (the tiled products and block inverses), through qt_rgf_solve_vb.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "E-points/s (RGF) and GW-SCBA time-to-converge at 1e-6 err, vs plain FP64 GPU"
NX, NM, NK, NE = 100, 128, 16, 4096
SEED = 2024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch-energies", type=int, default=64,
                    help="energies per step (x 16 k-points)")
    ap.add_argument("--fp64-energies", type=int, default=64,
                    help="energies (x 16 k) of the strided accuracy sample (every "
                         "4096/n-th energy), solved in FP64 and both split modes; 0 skips it")
    ap.add_argument("--hi-energies", type=int, default=16,
                    help="uneven workload: energies (x 8 k) of the complex128 split sample")
    ap.add_argument("--cpu-points", type=int, default=16)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-scba", action="store_true", help="skip the GW-SCBA mixing comparison")
    ap.add_argument("--scba-size", default="10,16,256",
                    help="slabs,orbitals,energies of the GW-SCBA device family")
    ap.add_argument("--scba-train", type=int, default=8,
                    help="training seeds of the learned mixer (disorder realisations)")
    ap.add_argument("--scba-test", type=int, default=2, help="held-out seeds")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-uneven", action="store_true",
                    help="skip the uneven-block sample of the default line")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the library's default wave size instead of autotuning it")
    ap.add_argument("--wave", type=int, default=0,
                    help="points per wave, set without autotuning (0: autotune unless --no-tune)")
    ap.add_argument("--workload", default="batched",
                    choices=["batched", "uneven", "gw", "scba"],
                    help="batched: 100 x 128 slabs (the headline); uneven: the 4000-atom graph; "
                         "gw: GW-SCBA on the 80-slab x 96-orbital device with 2048 energies; "
                         "scba: the plain / Pulay / learned mixing comparison alone "
                         "(--scba-size, --scba-train, --scba-test)")
    ap.add_argument("--gw-size", default="80,96,2048",
                    help="slabs,orbitals,energies of the --workload gw device")
    ap.add_argument("--gw-precisions", default="mixed-fp64,mixed",
                    help="--workload gw: split precisions to converge (each checked in FP64)")
    ap.add_argument("--gw-max-iter", type=int, default=60)
    ap.add_argument("--gw-tol", type=float, default=1e-8)
    return ap.parse_args()


def device():
    from quantum_transport_gb300.devices import config_batched
    return config_batched(seed=SEED, nE=NE, nk=NK, nx=NX, nm=NM)


def config_dict(a, extra=None):
    c = {"workload": "batched RGF, 100 slabs x 128 orbitals, 16 k x 4096 E "
                     "(65,536 (E,k) solves), seeded synthetic chain",
         "slabs": NX, "orbitals_per_slab": NM, "k_points": NK, "energies": NE,
         "points_per_step": a.batch_energies * NK,
         "outputs": "T(E) Caroli, tr, tre, diag G^R (LDOS), diag G^<",
         "sancho_tol": 1e-10, "eta_lead": 1e-5,
         "l2": "no flush: per-step working set (g_l, g^<_l per point x slabs) >> 129 MB L2"}
    if extra:
        c.update(extra)
    return c


class Clocks:
    """nvidia-smi sampling during the timed region (SM clock, throttle reasons)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) > 8
                          for i, v in enumerate(r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def cpu_baseline(dev, npts, threads):
    """The C restatement on the host cores: npts points of the same workload."""
    from oracle import cref
    cref.build()
    ne = max(1, npts // NK)
    t0 = time.perf_counter()
    r = cref.rgf(dev.H00, dev.H10, dev.E[:ne], NX, mul=0.1, mur=-0.1, templ=300.0, tempr=300.0,
                 sancho_tol=1e-10, threads=threads, want_diag=True)
    dt = time.perf_counter() - t0
    return ne * NK / dt, dt, r


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    dev = device()
    threads = os.cpu_count() or 1
    npts = max(NK, (threads // NK) * NK) if threads >= NK else NK
    for _ in range(a.warmup):
        cpu_baseline(dev, npts, threads)
    times = []
    for _ in range(a.steps):
        _, dt, _ = cpu_baseline(dev, npts, threads)
        times.append(dt)
    ms = 1e3 * sum(times) / len(times)
    v = npts / (ms / 1e3)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "E-points/s",
            "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic (seeded)",
            "config": config_dict(a, {"points_per_step": npts}),
            "cpu_baseline": {"value": v, "unit": "E-points/s", "cores": threads, "kind": "port",
                             "sample": f"{npts} points (one energy x 16 k) per step of the same "
                                       "workload; C99+OpenMP restatement of the reference sweep "
                                       "(no Fortran compiler on the box)"},
            "e2e": {"value": v, "unit": "E-points/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def scba_comparison(ctx, a):
    """GW-SCBA to residual 1e-8 with plain (the reference's linear mixing), Pulay and learned
    mixing on held-out seeds of the disorder family; the learned mixer is trained here first,
    on the GPU with the library's kernels, from the method's own iterates."""
    from quantum_transport_gb300 import gw, mixing
    from quantum_transport_gb300.devices import disordered_gw_device
    nx, nm, nE = (int(x) for x in a.scba_size.split(","))

    def system(seed, precision="fp64"):
        d = disordered_gw_device(seed, nx=nx, nm=nm, nE=nE)
        return gw.GwSystem(ctx, d.H00, d.H10, d.E, d.nx, d.V, mu=(0.1, -0.1),
                           precision=precision)

    train_sys = [system(100 + i) for i in range(a.scba_train)]
    test_sys = [system(900 + i) for i in range(a.scba_test)]
    t0 = time.perf_counter()
    mixer = mixing.LearnedMixer(ctx, nE, seed=5, max_batch=max(2048, nx * nm))
    X, T, fps, _ = mixing.collect(train_sys)
    mixing.train(mixer, X, T, steps=800, batch=2048, lr=1e-3)
    X2, T2, _, _ = mixing.collect(train_sys, mixer=mixer, fixed_points=fps)
    mixing.train(mixer, np.concatenate([X, X2]), np.concatenate([T, T2]), steps=800,
                 batch=2048, lr=5e-4, seed=1)
    t_train = time.perf_counter() - t0
    out = {m: {"evaluations": [], "seconds": [], "converged": []}
           for m in ("plain", "pulay", "learned")}
    diff = 0.0
    for s in test_sys:
        runs = {m: mixing.run_scba(s, method=m, mixer=mixer if m == "learned" else None,
                                   tol=1e-8, max_iter=200) for m in out}
        for m, r in runs.items():
            out[m]["evaluations"].append(r.evaluations)
            out[m]["seconds"].append(r.seconds)
            out[m]["converged"].append(r.residuals[-1] <= 1e-8)
        for x, y in zip(runs["learned"].sigma, runs["plain"].sigma):
            diff = max(diff, float((x - y).abs().max() / y.abs().max()))
    # plain-mixing SCBA to residual 1e-6 in FP64 and in both split precisions on one held-out
    # seed: time to converge, and the errors in terminal current and LDOS against FP64
    runs = {}
    for p in ("fp64", "mixed-fp64", "mixed"):
        s = system(900, p)
        s.scba(alpha=0.3, tol=1e-6, max_iter=2)  # first-call set-up
        t0 = time.perf_counter()
        SR, SL, _, res, cur = s.scba(alpha=0.3, tol=1e-6, max_iter=200, with_currents=True)
        dt = time.perf_counter() - t0
        ob = s.currents(SR, SL)
        runs[p] = (dt, len(res), float(res[-1]), cur[-1], -2.0 * ob["diag_gr"].imag)
    t64, n64, r64, c64, l64 = runs["fp64"]
    precision = {"fp64": {"seconds": t64, "iterations": n64, "final_residual": r64,
                          "current_A": [float(x) for x in c64]}}
    for p in ("mixed-fp64", "mixed"):
        t, nit, rr, c, ld = runs[p]
        precision[p] = {"seconds": t, "iterations": nit, "final_residual": rr,
                        "time_vs_fp64": t / t64,
                        "current_rel_err": float(np.max(np.abs(c - c64) / np.abs(c64))),
                        "ldos_rel_err": float(np.abs(ld - l64).max() / np.abs(l64).max())}
    mean = lambda v: float(np.mean(v))
    return {"workload": f"GW-SCBA, {nx} slabs x {nm} orbitals x {nE} energies, on-site disorder "
                        "sigma ~ U[0.05, 0.3] eV, V_ij = 14.4/(|r_i - r_j| + 1) eV, residual <= 1e-8",
            "train_seeds": len(train_sys), "test_seeds": len(test_sys),
            "training_seconds": t_train,
            **{m: {"evaluations": mean(v["evaluations"]),
                   "evaluations_median": float(np.median(v["evaluations"])),
                   "seconds": mean(v["seconds"]), "converged": int(sum(v["converged"]))}
               for m, v in out.items()},
            "learned_faster_than_pulay_seeds": int(sum(
                x < y for x, y in zip(out["learned"]["seconds"], out["pulay"]["seconds"]))),
            "learned_vs_plain_time": mean(out["learned"]["seconds"]) / mean(out["plain"]["seconds"]),
            "learned_vs_pulay_time": mean(out["learned"]["seconds"]) / mean(out["pulay"]["seconds"]),
            "fixed_point_max_rel_diff": diff,
            "precision_to_1e-6": precision}


def _point_errors(x, ref, per_point):
    """max and median over points of max|x - ref| / max|ref| within each point."""
    d = np.abs(x - ref).reshape(-1, per_point).max(axis=1)
    m = np.abs(ref).reshape(-1, per_point).max(axis=1)
    r = d / np.maximum(m, 1e-300)
    return float(r.max()), float(np.median(r))


def uneven_sample(ctx, n_energies=64, n_fp64=16):
    """The uneven-block configuration beside the headline: the 4000-atom graph device
    (25 slabs of 134-184 orbitals, 8 k) through the variable-block sweep.  Both split modes
    solve n_energies energies spread over the [-2, 2] eV window x 8 k in one wave (timed
    with CUDA events after a one-energy warm-up call); the FP64 path solves every
    (n_energies / n_fp64)-th of them, which gives its throughput and the T(E) errors."""
    import torch
    from quantum_transport_gb300 import rgf
    from quantum_transport_gb300.devices import config_uneven
    d = config_uneven()
    nk = len(d.kpts)
    sizes = np.array(d.sizes, dtype=np.int32)
    hii, hoff, _ = rgf.pack_blocks(d.Hii, nk)
    h1i, h1off, _ = rgf.pack_blocks(d.H1i, nk)
    Hd, H1d = torch.from_numpy(hii).cuda(), torch.from_numpy(h1i).cuda()
    Eall = torch.from_numpy(d.E).cuda()
    Es = Eall[::len(d.E) // n_energies][:n_energies].contiguous()
    sub = n_energies // n_fp64
    E64 = Es[::sub].contiguous()
    kw = dict(mul=0.1, mur=-0.1, templ=300.0, tempr=300.0, sancho_tol=1e-10,
              sancho_max_iter=100, caroli=True)
    stream = torch.cuda.current_stream()

    def solve(prec, E, ne):
        o = {"T": torch.zeros(ne * nk, dtype=torch.float64, device="cuda"),
             "status": torch.zeros(ne * nk, dtype=torch.int32, device="cuda")}
        rgf.rgf_variableblock_device(ctx, sizes, Hd, hoff, H1d, h1off, nk, E, 1, o,
                                     precision=prec, **kw)  # first-call set-up
        ctx.sync()
        ctx.inverse_fallbacks(reset=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rgf.rgf_variableblock_device(ctx, sizes, Hd, hoff, H1d, h1off, nk, E, ne, o,
                                     precision=prec, **kw)
        e1.record(stream)
        e1.synchronize()
        ctx.sync()
        return (ne * nk / (e0.elapsed_time(e1) / 1e3), o["T"].cpu().numpy(),
                int((o["status"] != 0).sum().item()), ctx.inverse_fallbacks())

    v64, T64, bad64, _ = solve("fp64", E64, E64.numel())
    out = {"workload": f"uneven-block RGF, 4000-atom random graph sliced into {len(sizes)} slabs "
                       f"of {sizes.min()}-{sizes.max()} orbitals, {nk} k; {n_energies} energies "
                       f"across [-2, 2] eV per split-mode wave, every {sub}th in FP64",
           "fp64": {"value": v64, "unit": "E-points/s", "points": int(T64.size),
                    "points_bad_status": bad64}}
    for prec in ("mixed-fp64", "mixed"):
        v, T, bad, fb = solve(prec, Es, n_energies)
        Tm = T.reshape(n_energies, nk)[::sub].reshape(-1)
        err = np.abs(Tm - T64)
        out[prec] = {"value": v, "unit": "E-points/s", "points": int(T.size),
                     "speedup_vs_fp64": v / v64,
                     "T_rel_err_max": float(err.max() / np.abs(T64).max()),
                     "T_rel_err_median": float(np.median(err) / np.abs(T64).max()),
                     "points_bad_status": bad, "inverses_redone_fp64": fb}
    return out


def accuracy_sample(ctx, H00, H10, E, nm2, kw, n_energies, split_value):
    """FP64-pipe path against both split precisions on a strided sample of the workload:
    every (NE / n_energies)-th energy across the whole [-2, 2] eV window x 16 k.  Reports
    the FP64 path's throughput, the complex128 split mode's throughput, and for both split
    modes the max and median over points of the relative errors in T(E), LDOS
    (-2 Im diag G^R per orbital) and diag G^<.  Returns (report, FP64 T per point)."""
    import torch
    from quantum_transport_gb300 import rgf
    stride = max(1, NE // n_energies)
    Es = E[::stride].contiguous()
    ne = Es.numel()
    Pf = ne * NK
    per = NX * NM

    def outputs():
        return {"T": torch.zeros(Pf, dtype=torch.float64, device="cuda"),
                "tr": torch.zeros(Pf, dtype=torch.float64, device="cuda"),
                "tre": torch.zeros(Pf, dtype=torch.float64, device="cuda"),
                "diag_gr": torch.zeros(Pf * per, dtype=torch.complex128, device="cuda"),
                "diag_gl": torch.zeros(Pf * per, dtype=torch.complex128, device="cuda"),
                "status": torch.zeros(Pf, dtype=torch.int32, device="cuda")}
    res, secs = {}, {}
    for prec in ("fp64", "mixed-fp64", "mixed"):
        o = outputs()
        rgf.rgf_solve_device(ctx, H00, nm2, 0, H10, 0, 0, NM, NX, NK, Es, 1, o,
                             precision=prec, **kw)  # first-call set-up
        ctx.sync()
        t0 = time.perf_counter()
        rgf.rgf_solve_device(ctx, H00, nm2, 0, H10, 0, 0, NM, NX, NK, Es, ne, o,
                             precision=prec, **kw)
        ctx.sync()
        secs[prec] = time.perf_counter() - t0
        res[prec] = {k: v.cpu().numpy() for k, v in o.items()}
    r64 = res["fp64"]
    v64 = Pf / secs["fp64"]
    # conditioning: where the FP64-grade split mode and the FP64 path (two correct FP64-grade
    # operation orders) differ in T by more than 1e-8, the point is ill conditioned (a
    # transverse channel opening at eta = 1e-5)
    eh = np.abs(res["mixed-fp64"]["T"] - r64["T"]) / np.abs(r64["T"])
    good = eh <= 1e-8
    Eh = Es.cpu().numpy()
    out = {"value": v64, "unit": "E-points/s", "sample_points": Pf,
           "sample": f"energies E[::{stride}] ({ne} across [-2, 2] eV) x {NK} k",
           "speedup_split_vs_fp64": split_value / v64,
           "points_bad_status": int((r64["status"] != 0).sum()),
           "ill_conditioned_points": [{"E_eV": float(Eh[i // NK]), "k_index": int(i % NK),
                                       "T_fp64": float(r64["T"][i]),
                                       "T_rel_diff_fp64_grade": float(eh[i])}
                                      for i in np.flatnonzero(~good)]}
    for prec in ("mixed", "mixed-fp64"):
        r = res[prec]
        tre = np.abs(r["T"] - r64["T"]) / np.abs(r64["T"])
        lmax, lmed = _point_errors(r["diag_gr"].imag, r64["diag_gr"].imag, per)
        gmax, gmed = _point_errors(r["diag_gl"], r64["diag_gl"], per)
        e = {"T_rel_err_max": float(tre.max()), "T_rel_err_median": float(np.median(tre)),
             "T_rel_err_max_well_conditioned": float(tre[good].max()),
             "T_err_max_vs_peak": float(np.abs(r["T"] - r64["T"]).max() / np.abs(r64["T"]).max()),
             "ldos_rel_err_max": lmax, "ldos_rel_err_median": lmed,
             "diag_glesser_rel_err_max": gmax, "diag_glesser_rel_err_median": gmed,
             "points_bad_status": int((r["status"] != 0).sum())}
        if prec == "mixed":
            out.update(e)
        else:
            out["mixed_fp64"] = {"value": Pf / secs[prec], "unit": "E-points/s",
                                 "sample_points": Pf, "speedup_vs_fp64": (Pf / secs[prec]) / v64,
                                 **e}
    return out, r64["T"]


def run_ours(a):
    import torch
    import torch.distributed as dist

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", rank=rank, world_size=world)

    def barrier():
        if world > 1:
            dist.barrier()

    from quantum_transport_gb300.build import build
    build()
    from quantum_transport_gb300 import rgf
    from quantum_transport_gb300.shard import energy_range, max_over_ranks

    dev = device()
    ctx = rgf.Context(local)
    B = a.batch_energies
    P = B * NK
    nblk = NE // B
    cm = lambda x: torch.from_numpy(rgf.colmajor(x)).cuda()
    H00 = cm(dev.H00)                 # (16, 128, 128) complex128, column-major per block
    H10 = cm(dev.H10)
    E = torch.from_numpy(dev.E).cuda()
    nm2 = NM * NM
    out = {"T": torch.zeros(P, dtype=torch.float64, device="cuda"),
           "tr": torch.zeros(P, dtype=torch.float64, device="cuda"),
           "tre": torch.zeros(P, dtype=torch.float64, device="cuda"),
           "diag_gr": torch.zeros(P * NX * NM, dtype=torch.complex128, device="cuda"),
           "diag_gl": torch.zeros(P * NX * NM, dtype=torch.complex128, device="cuda"),
           "status": torch.zeros(P, dtype=torch.int32, device="cuda")}
    kw = dict(mul=0.1, mur=-0.1, templ=300.0, tempr=300.0, sancho_tol=1e-10, caroli=True)

    # each rank owns a contiguous block of the energy grid and cycles through it
    lo, hi = energy_range(NE, world, rank)
    nblk_r = max(1, (hi - lo) // B)

    def step(i, precision="mixed", o=out, nE=B):
        e0 = min(lo + (i % nblk_r) * B, NE - B)
        rgf.rgf_solve_device(ctx, H00, nm2, 0, H10, 0, 0, NM, NX, NK, E[e0:], nE, o,
                             precision=precision, **kw)

    torch.cuda.synchronize()
    # batch schedule: points per wave, measured on this workload before the warm-up
    wave, wave_ms = a.wave, {}
    if a.wave:
        ctx.set_wave_points(a.wave)
    elif not a.no_tune:
        from quantum_transport_gb300 import autotune
        wave, wave_ms = autotune.tune_wave(ctx, lambda: step(0), P, nk=NK)
    for i in range(a.warmup):
        step(i)
    ctx.sync()
    stream = torch.cuda.current_stream()  # the context launches on torch's current stream
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = Clocks(local)
    ctx.profile_read()  # drop warm-up entries
    ctx.profile(True)
    n0 = rgf.kernel_launches()
    ctx.inverse_fallbacks(reset=True)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0.record(stream)
    for i in range(a.steps):
        step(a.warmup + i)
    ev1.record(stream)
    ev1.synchronize()
    ctx.sync()
    clk = clocks.stop()
    launches = rgf.kernel_launches() - n0
    ctx.profile(False)
    prof = ctx.profile_read()
    ms = ev0.elapsed_time(ev1) / a.steps
    ms = max_over_ranks(ms)
    status_bad = int((out["status"] != 0).sum().item())
    value = world * P / (ms / 1e3)

    pk, pk_kind = peaks()
    tot_ms = sum(v[1] for v in prof.values()) or 1.0
    dom = prof.get("zgemm_oz_c64", (0, 0.0, 0.0, 0.0))
    alg_tf = dom[2] / (dom[1] / 1e3) / 1e12 if dom[1] else 0.0
    exe_tf = dom[3] / (dom[1] / 1e3) / 1e12 if dom[1] else 0.0
    peak = pk.get("bf16_tflops_sustained", pk.get("bf16_tflops"))
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp) and dom[0]:
        with open(tp) as f:
            bpp = json.load(f).get("zgemm_c64_tma_dram_bytes_per_product")
        if bpp:
            traffic = bpp * (dom[2] / (8.0 * NM ** 3)) / dom[0]
    roofline = {"kernel": "zgemm_c64_tma_kernel (complex64 4-digit split product, TMA-fed)",
                "bound": "tensor", "achieved": alg_tf, "peak": peak, "unit": "TFLOP/s",
                "frac": alg_tf / peak if peak else None, "traffic": traffic,
                "peak_source": f"bf16_tflops_sustained of {pk_kind}",
                "achieved_is": "algorithmic 8 n^3 flops per complex block product / event time",
                "executed_tensor_tflops": exe_tf,
                "executed_frac": exe_tf / peak if peak else None,
                "launches": dom[0], "avg_launch_ms": dom[1] / dom[0] if dom[0] else None,
                "time_share": {k: round(v[1] / tot_ms, 4) for k, v in prof.items()}}
    line = {"metric": METRIC, "value": value, "unit": "E-points/s", "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16-digit split (c64 sweep, "
            "FP64-grade c128 leads)", "data": "synthetic (seeded, no dataset)",
            "config": config_dict(a, {"parallelism": f"points sharded over {world} GPU(s)",
                                      "points_bad_status": status_bad,
                                      "inverses_redone_fp64": ctx.inverse_fallbacks(),
                                      "wave_points": wave or "library default (608)",
                                      "wave_tuning_ms_per_call": {str(k): round(v, 2) for k, v
                                                                  in wave_ms.items()}}),
            "roofline": roofline, "clocks": clk, "gpu_launches": launches}

    T64 = None
    if rank == 0 and a.fp64_energies > 0:
        # the sample starts at E[0]: its first 16 points are the CPU baseline's points
        line["fp64_gpu"], T64 = accuracy_sample(ctx, H00, H10, E, nm2, kw, a.fp64_energies,
                                                value / world)
    if rank == 0 and not a.no_scba:
        line["scba"] = scba_comparison(ctx, a)
    if rank == 0 and not a.no_uneven:
        line["uneven"] = uneven_sample(ctx)
    if rank == 0:
        if world == 1 and not a.no_cpu:
            threads = os.cpu_count() or 1
            v, dt, r = cpu_baseline(dev, a.cpu_points, threads)
            line["cpu_baseline"] = {"value": v, "unit": "E-points/s", "cores": threads,
                                    "kind": "port",
                                    "sample": f"{max(1, a.cpu_points // NK) * NK} points (one "
                                              f"energy x 16 k) of the same workload, {dt:.1f} s; "
                                              "C99+OpenMP restatement of the reference sweep"}
            Tc = r["T"].ravel()
            if T64 is not None:
                line["cpu_baseline"]["T_rel_err_vs_fp64_gpu"] = float(
                    np.max(np.abs(Tc - T64[:Tc.size]) / np.abs(T64[:Tc.size])))
        if not a.no_e2e:
            # ---- end to end through the host-pointer C-ABI call
            Eh = dev.E
            rgf.rgf_solve(ctx, dev.H00, dev.H10, Eh[:B], NX, nk=NK, precision="mixed",
                          want_diag=True, **kw)
            t0 = time.perf_counter()
            ne = max(1, min(a.steps, 3))
            for i in range(ne):
                blk = (i + 1) % nblk
                r = rgf.rgf_solve(ctx, dev.H00, dev.H10, Eh[blk * B:(blk + 1) * B], NX, nk=NK,
                                  precision="mixed", want_diag=True, **kw)
            te = (time.perf_counter() - t0) / ne
            h2d = dev.H00.nbytes + dev.H10.nbytes + B * 8
            d2h = P * (3 * 8 + 4 + 8) + 3 * P * NX * NM * 16
            line["e2e"] = {"value": P / te, "unit": "E-points/s", "h2d_bytes_per_step": h2d,
                           "d2h_bytes_per_step": d2h, "steps": ne,
                           "points_bad_status": int((r["status"] != 0).sum())}
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


def run_uneven(a):
    """The uneven-block workload on one GPU: one step = ``--batch-energies`` energies x 8 k
    of the 4000-atom graph device through the variable-block sweep (complex64 split path),
    plus FP64 and complex128-split samples of the same points for the T(E) error."""
    import torch
    from quantum_transport_gb300.build import build
    build()
    from quantum_transport_gb300 import rgf
    from quantum_transport_gb300.devices import config_uneven
    d = config_uneven()
    nk, nEg = len(d.kpts), len(d.E)
    sizes = np.array(d.sizes, dtype=np.int32)
    hii, hoff, _ = rgf.pack_blocks(d.Hii, nk)
    h1i, h1off, _ = rgf.pack_blocks(d.H1i, nk)
    Hd, H1d = torch.from_numpy(hii).cuda(), torch.from_numpy(h1i).cuda()
    E = torch.from_numpy(d.E).cuda()
    ctx = rgf.Context(0)
    B = a.batch_energies
    P = B * nk
    dsum = int(sizes.sum())

    def outputs(p):
        return {"T": torch.zeros(p, dtype=torch.float64, device="cuda"),
                "tr": torch.zeros(p, dtype=torch.float64, device="cuda"),
                "tre": torch.zeros(p, dtype=torch.float64, device="cuda"),
                "diag_gr": torch.zeros(p * dsum, dtype=torch.complex128, device="cuda"),
                "diag_gl": torch.zeros(p * dsum, dtype=torch.complex128, device="cuda"),
                "status": torch.zeros(p, dtype=torch.int32, device="cuda")}
    out = outputs(P)
    kw = dict(mul=0.1, mur=-0.1, templ=300.0, tempr=300.0, sancho_tol=1e-10,
              sancho_max_iter=100, caroli=True)
    nblk = nEg // B

    def step(i, precision="mixed", o=out, nE=B, e0=None):
        e0 = (i % nblk) * B if e0 is None else e0
        rgf.rgf_variableblock_device(ctx, sizes, Hd, hoff, H1d, h1off, nk, E[e0:], nE, o,
                                     precision=precision, **kw)

    wave, wave_ms = a.wave, {}
    if a.wave:
        ctx.set_wave_points(a.wave)
    elif not a.no_tune:
        from quantum_transport_gb300 import autotune
        wave, wave_ms = autotune.tune_wave(ctx, lambda: step(0), P, nk=nk)
    for i in range(a.warmup):
        step(i)
    ctx.sync()
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = Clocks(0)
    ctx.profile_read()
    ctx.profile(True)
    n0 = rgf.kernel_launches()
    ctx.inverse_fallbacks(reset=True)
    torch.cuda.synchronize()
    clocks.start()
    ev0.record(stream)
    for i in range(a.steps):
        step(a.warmup + i)
    ev1.record(stream)
    ev1.synchronize()
    ctx.sync()
    clk = clocks.stop()
    launches = rgf.kernel_launches() - n0
    ctx.profile(False)
    prof = ctx.profile_read()
    ms = ev0.elapsed_time(ev1) / a.steps
    value = P / (ms / 1e3)
    flops = sum(120.0 * float(n) ** 3 for n in sizes)  # F_RGF per point, sum over slabs
    tot_ms = sum(v[1] for v in prof.values()) or 1.0
    dom = prof.get("zgemm_oz_c64", (0, 0.0, 0.0, 0.0))
    pk, pk_kind = peaks()
    peak = pk.get("bf16_tflops_sustained", pk.get("bf16_tflops"))
    alg_tf = dom[2] / (dom[1] / 1e3) / 1e12 if dom[1] else 0.0
    line = {"metric": METRIC, "value": value, "unit": "E-points/s", "n_gpus": 1,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16-digit split (c64 sweep, FP64-grade c128 leads)",
            "data": "synthetic (seeded random graph, no dataset)",
            "config": {"workload": f"uneven-block RGF, 4000-atom random graph in a 60 x 6 x 6 "
                                   f"A box sliced into {len(sizes)} slabs of {sizes.min()}-"
                                   f"{sizes.max()} orbitals, {nk} k x {nEg} E",
                       "points_per_step": P, "rgf_flop_per_point": flops,
                       "algorithmic_tflops": value * flops / 1e12,
                       "l2": "inputs and scratch per step exceed L2 (129 MB)",
                       "points_bad_status": int((out["status"] != 0).sum().item()),
                       "inverses_redone_fp64": ctx.inverse_fallbacks(),
                       "wave_points": wave or "library default (608)",
                       "wave_tuning_ms_per_call": {str(k): round(v, 2)
                                                   for k, v in wave_ms.items()}},
            "roofline": {"kernel": "zgemm_oz_kernel (complex64 split product, 128-row tiles)",
                         "bound": "tensor", "achieved": alg_tf, "peak": peak, "unit": "TFLOP/s",
                         "frac": alg_tf / peak if peak else None, "traffic": None,
                         "peak_source": f"bf16_tflops_sustained of {pk_kind}",
                         "launches": dom[0],
                         "time_share": {k: round(v[1] / tot_ms, 4) for k, v in prof.items()}},
            "clocks": clk, "gpu_launches": launches}
    # FP64 and complex128-split samples of the first points, and their T(E) errors
    samples = {}
    for prec, ne in (("fp64", a.fp64_energies), ("mixed-fp64", a.hi_energies)):
        if ne <= 0:
            continue
        o = outputs(ne * nk)
        step(0, prec, o, 1, e0=0)  # first-call set-up
        ctx.sync()
        t0 = time.perf_counter()
        step(0, prec, o, ne, e0=0)
        ctx.sync()
        samples[prec] = (o, ne * nk / (time.perf_counter() - t0))
    om = outputs(P)
    step(0, "mixed", om, B, e0=0)
    ctx.sync()
    Tm = om["T"].cpu().numpy()
    if "fp64" in samples:
        T64 = samples["fp64"][0]["T"].cpu().numpy()
        m = T64.size
        line["fp64_gpu"] = {"value": samples["fp64"][1], "unit": "E-points/s",
                            "sample_points": m,
                            "speedup_split_vs_fp64": value / samples["fp64"][1],
                            "T_rel_err_max_vs_peak": float(np.abs(Tm[:m] - T64).max() /
                                                           np.abs(T64).max())}
        if "mixed-fp64" in samples:
            Th = samples["mixed-fp64"][0]["T"].cpu().numpy()
            k = min(m, Th.size)
            line["fp64_gpu"]["mixed_fp64"] = {
                "value": samples["mixed-fp64"][1], "unit": "E-points/s",
                "sample_points": Th.size,
                "T_rel_err_max_vs_peak": float(np.abs(Th[:k] - T64[:k]).max() /
                                               np.abs(T64[:k]).max())}
    if not a.no_e2e:
        r = rgf.rgf_variableblock_forward(ctx, d.Hii, d.H1i, d.E[:B], nk=nk, precision="mixed",
                                          **kw)  # first call
        t0 = time.perf_counter()
        r = rgf.rgf_variableblock_forward(ctx, d.Hii, d.H1i, d.E[B:2 * B], nk=nk,
                                          precision="mixed", **kw)
        te = time.perf_counter() - t0
        line["e2e"] = {"value": P / te, "unit": "E-points/s",
                       "h2d_bytes_per_step": int(hii.nbytes + h1i.nbytes + B * 8),
                       "d2h_bytes_per_step": int(P * (3 * 8 + 4 + 8) + 3 * P * dsum * 16),
                       "steps": 1, "points_bad_status": int((r["status"] != 0).sum())}
    print(json.dumps(line), flush=True)
    ctx.close()


def run_gw(a):
    """GW-SCBA at size: plain linear mixing (alpha = 0.3, the reference's scheme) to residual
    --gw-tol on a seeded 80-slab x 96-orbital chain (H_ii shared by all slabs: on-site
    U[-1, 1] eV, off-diagonal N(0, 0.1) eV; H_i,i+1 = -2.7 I + N(0, 0.05)), 2048 energies
    on [-4, 4] eV, V_ij = 14.4 / (|r_i - r_j| + 1) eV on a 0.25 nm grid, FFT length 4096.

    Each split precision runs to convergence in turn (the device holds one SCBA at a time:
    the three self-energies and the map's six arrays, 24 GB each).  Its fixed point S* is
    then checked in FP64, which would take about 45 minutes to converge itself:
      - one FP64 evaluation of the map at S*: its residual ||F64(S*) - S*|| / ||F64(S*)||
        and its time (the FP64 seconds per iteration);
      - the FP64 RGF at S*: terminal currents and LDOS against the split RGF's at S*.
    The FP64 time to converge is projected as the split run's iteration count times the
    FP64 seconds per iteration, and labelled so."""
    import torch
    from quantum_transport_gb300.build import build
    build()
    from quantum_transport_gb300 import gw, rgf
    from quantum_transport_gb300.devices import coulomb_block, make_chain_device
    nx, nm, nE = (int(x) for x in a.gw_size.split(","))
    d = make_chain_device(nx, nm, nE, -4.0, 4.0, seed=SEED)
    V = coulomb_block(nm)
    ctx = rgf.Context(0)
    precs = [p for p in a.gw_precisions.split(",") if p != "fp64"]
    out = {}
    clocks = Clocks(0)
    clocks.start()
    s64 = gw.GwSystem(ctx, d.H00[0], d.H10, d.E, nx, V, mu=(0.1, -0.1), precision="fp64")
    for p in precs:
        s = gw.GwSystem(ctx, d.H00[0], d.H10, d.E, nx, V, mu=(0.1, -0.1), precision=p)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        SR, SL, SG, res, cur = s.scba(alpha=0.3, tol=a.gw_tol, max_iter=a.gw_max_iter,
                                      with_currents=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        it6 = next((i + 1 for i, r in enumerate(res) if r <= 1e-6), None)
        e = {"seconds": dt, "iterations": int(len(res)),
             "seconds_per_iteration": dt / max(1, len(res)),
             "iterations_to_1e-6": it6,
             "seconds_to_1e-6": None if it6 is None else it6 * dt / len(res),
             "final_residual": float(res[-1]), "converged": bool(res[-1] <= a.gw_tol),
             "residuals": [float(x) for x in res],
             "current_A": [float(x) for x in cur[-1]]}
        # the split RGF and the FP64 RGF at the same S* (each timed: the RGF's share of an
        # iteration)
        t0 = time.perf_counter()
        ob = s.currents(SR, SL)
        t_rgf = time.perf_counter() - t0
        t0 = time.perf_counter()
        o64 = s64.currents(SR, SL)
        t_rgf64 = time.perf_counter() - t0
        ld, ld64 = -2.0 * ob["diag_gr"].imag, -2.0 * o64["diag_gr"].imag
        e["rgf_at_fixed_point"] = {
            "seconds": t_rgf, "fp64_seconds": t_rgf64,
            "tr_rel_err": float(np.abs(ob["tr"] - o64["tr"]).max() / np.abs(o64["tr"]).max()),
            "tre_rel_err": float(np.abs(ob["tre"] - o64["tre"]).max() /
                                 np.abs(o64["tre"]).max()),
            "ldos_rel_err": float(np.abs(ld - ld64).max() / np.abs(ld64).max())}
        del s
        torch.cuda.empty_cache()
        # one FP64 map at S* (in place: S becomes the FP64 iterate mixed with S*)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, _, _, r64, c64 = s64.scba(alpha=0.3, tol=0.0, max_iter=1, start=(SR, SL, SG),
                                     with_currents=True)
        torch.cuda.synchronize()
        t64 = time.perf_counter() - t0
        e["fp64_map_at_fixed_point"] = {
            "residual": float(r64[0]), "seconds": t64,
            "current_A": [float(x) for x in c64[0]],
            "current_rel_err": float(np.max(np.abs(np.array(e["current_A"]) - c64[0]) /
                                            np.abs(c64[0])))}
        if it6 is not None:
            e["fp64_seconds_to_1e-6_projected"] = it6 * t64
            e["speedup_vs_fp64_to_1e-6"] = it6 * t64 / e["seconds_to_1e-6"]
        out[p] = e
        del SR, SL, SG
        torch.cuda.empty_cache()
    clk = clocks.stop()
    L = 1 << int(np.ceil(np.log2(2 * nE)))
    line = {"metric": METRIC, "workload": "gw", "unit": "s to residual", "tol": a.gw_tol,
            "higher_is_better": False, "n_gpus": 1, "data": "synthetic (seeded, no dataset)",
            "config": {"workload": f"GW-SCBA, {nx} slabs x {nm} orbitals x {nE} energies on "
                                   f"[-4, 4] eV, plain linear mixing alpha = 0.3 to residual "
                                   f"{a.gw_tol:g} (max {a.gw_max_iter} iterations), FFT length {L}",
                       "memory": "the three Sigma arrays + six [nE][nx][nm^2] complex128 "
                                 "arrays in the map (G, then P -> W in place, Sigma_new over "
                                 f"G): {9 * nE * nx * nm * nm * 16 / 1e9:.0f} GB",
                       "fp64_reference": "one FP64 map and the FP64 RGF at each split fixed "
                                         "point; FP64 time to converge projected"},
            "runs": out, "clocks": clk}
    print(json.dumps(line), flush=True)
    ctx.close()


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "uneven":
        run_uneven(a)
    elif a.workload == "gw":
        run_gw(a)
    elif a.workload == "scba":
        from quantum_transport_gb300.build import build
        build()
        from quantum_transport_gb300 import rgf
        ctx = rgf.Context(0)
        print(json.dumps({"metric": METRIC, "workload": "scba",
                          "scba": scba_comparison(ctx, a)}), flush=True)
        ctx.close()
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
