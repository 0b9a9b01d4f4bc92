"""Batch-schedule autotuner for the batched sweeps.

The sweeps solve their (E, k) points in waves: every batched launch (block products,
inverses, decimation steps) covers the points of one wave. The wave size trades launch
count and per-launch prologues against the tail of the last round of work items on the
SMs. The library's default is 4 work items per SM (608 points on 152 SMs). ``tune_wave``
measures candidate sizes on the caller's own workload and sets the fastest on the context
(``qt_ctx_set_wave_points``). Results do not depend on the wave size; only the time does.
"""
from __future__ import annotations

import json
import os


def candidates(npts, nk=1, sms=None):
    """Wave sizes to try for calls of ``npts`` points: 2 to 8 work items per SM and one wave
    for the whole call, rounded down to whole energies (multiples of ``nk``)."""
    if sms is None:
        import torch
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    out = []
    for per_sm in (2, 3, 4, 5, 6, 8):
        out.append(min(per_sm * sms, npts))
    out.append(npts)
    out = sorted({max(nk, (p // nk) * nk) for p in out})
    return out


def tune_wave(ctx, run, npts, nk=1, cands=None, cache=None, key=None):
    """Time ``run()`` (one call of the workload, ``npts`` points, on ``ctx``) at each
    candidate wave size: one untimed call (scratch growth), then one call timed with CUDA
    events on the context's stream. Sets the fastest size on ``ctx`` and returns
    ``(best, {size: ms})``.

    With ``cache`` (a JSON file path) and ``key`` (a string naming the workload), a size
    measured before for the same GPU model and key is reused without timing."""
    import torch
    gpu = torch.cuda.get_device_name(torch.cuda.current_device())
    ckey = f"{gpu}|{key}" if key is not None else None
    if cache and ckey and os.path.exists(cache):
        with open(cache) as f:
            hit = json.load(f).get(ckey)
        if hit:
            ctx.set_wave_points(hit["best"])
            return hit["best"], {int(k): v for k, v in hit["ms"].items()}
    cands = list(cands) if cands is not None else candidates(npts, nk)
    stream = torch.cuda.current_stream()
    times = {}
    for P in cands:
        ctx.set_wave_points(P)
        run()
        ctx.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run()
        e1.record(stream)
        e1.synchronize()
        ctx.sync()
        times[P] = e0.elapsed_time(e1)
    best = min(times, key=times.get)
    ctx.set_wave_points(best)
    if cache and ckey:
        data = {}
        if os.path.exists(cache):
            with open(cache) as f:
                data = json.load(f)
        data[ckey] = {"best": best, "ms": times}
        with open(cache, "w") as f:
            json.dump(data, f, indent=1)
    return best, times
