"""Launch-shape autotuner.

Times candidate launch shapes of a kernel on the actual problem with CUDA
events (after warm-up), keeps the fastest, and caches the choice per device
name and problem size class in a JSON file ($ODIL_GB300_TUNE_CACHE, default
~/.cache/odil_gb300/autotune.json).
"""
import json
import os
import statistics

import torch

from ._capi import ODIL_ERR_SHAPE, OdilError


def _cache_path():
    return os.environ.get(
        "ODIL_GB300_TUNE_CACHE",
        os.path.join(os.path.expanduser("~"), ".cache", "odil_gb300",
                     "autotune.json"))


def _load():
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(data):
    path = _cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def _pow2_bucket(n):
    b = 1
    while b < n:
        b *= 2
    return b


def default_batch_march(max_nx):
    """Heuristic shape: 2 columns per thread, 16 prefetched rows."""
    cpt = 1 if max_nx <= 128 else (2 if max_nx <= 2048 else 4)
    threads = max(32, ((max_nx + cpt - 1) // cpt + 31) // 32 * 32)
    return {"threads": threads, "cpt": cpt, "pf": 16, "blocks_per_sm": 2}


def default_batch_solve(max_nx):
    """Heuristic shape of the persistent whole-batch solve: two columns per
    thread up to 1024 columns, else 4 (at most 512 threads with more than
    one column), 8 ring rows, 4 blocks per SM (the fastest measured on the
    512-instance batch, sides 64-512)."""
    cpt = 2 if max_nx <= 1024 else 4
    threads = max(32, ((max_nx + cpt - 1) // cpt + 31) // 32 * 32)
    return {"threads": threads, "cpt": cpt, "pf": 8, "blocks_per_sm": 4}


def candidates_batch_march(max_nx, smem_limit=200 * 1024):
    out = []
    for cpt in (1, 2, 4):
        threads = ((max_nx + cpt - 1) // cpt + 31) // 32 * 32
        if threads > 1024:
            continue
        for pf in (8, 16):
            smem = pf * max_nx * 4 + 512
            if smem > smem_limit:
                continue
            for bps in (1, 2, 4, 8):
                if bps * smem > 228 * 1024 or bps * threads > 2048:
                    continue
                out.append({"threads": threads, "cpt": cpt, "pf": pf,
                            "blocks_per_sm": bps})
    return out


def _time(fn, reps=3):
    st = torch.cuda.current_stream()
    fn()
    ts = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        fn()
        e1.record(st)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    return statistics.median(ts)


def tune_batch_march(batch, cache=True):
    dev = torch.cuda.get_device_name(batch.device)
    key = "wave_batch_march|%s|nx%d|n%d" % (dev, _pow2_bucket(batch.max_nx),
                                              _pow2_bucket(batch.n))
    data = _load() if cache else {}
    if key in data:
        return data[key]["cfg"]
    best = None
    results = []
    for cfg in candidates_batch_march(batch.max_nx):
        t = _time(lambda: batch.march(batch.rhs, batch.d, cfg))
        results.append((t, cfg))
        if best is None or t < best[0]:
            best = (t, cfg)
    if cache:
        data[key] = {"cfg": best[1], "ms": best[0],
                     "tried": [[t, c] for t, c in results]}
        _store(data)
    return best[1]


def march_max_threads(cpt, pf):
    """Block limit of the FP32 march (register ring of cpt * pf values)."""
    b = cpt * pf * 4
    return 1024 if b <= 64 else (512 if b <= 128 else 256)


# (cpt, halo, pf, exchange) of the cluster-tiled march (exchange 0: cluster
# barrier and reload from global memory; 1: pushes into the neighbours'
# shared memory).
TILED_SHAPES = ((4, 32, 16, 0), (4, 48, 16, 0), (8, 96, 16, 0),
                (2, 16, 16, 1), (4, 8, 8, 1), (4, 16, 16, 1), (4, 24, 8, 1),
                (4, 32, 16, 1), (8, 32, 16, 1), (8, 64, 16, 1))


def candidates_march(nx, dtype=torch.float32):
    """Single-block shapes (FP32; the FP64 entry point's own shape) and
    cluster-tiled shapes with at most 16 blocks."""
    out = []
    if dtype == torch.float32:
        for cpt in (1, 2, 4, 8):
            threads = ((nx + cpt - 1) // cpt + 31) // 32 * 32
            if cpt > 1 and (nx + cpt - 1) // cpt < 32:
                continue
            for pf in (8, 16):
                if threads <= march_max_threads(cpt, pf):
                    out.append({"kind": "block", "cpt": cpt, "pf": pf})
    elif nx <= 2048:
        out.append({"kind": "default"})
    if nx >= 2:
        for cpt, halo, pf, exch in TILED_SHAPES:
            if dtype == torch.float64 and cpt * pf > 64:
                continue  # register ring too large for FP64
            tiles = -(-nx // (32 * cpt - 2 * halo))
            for warps in (1, 2, 4):
                if (warps > 1 and warps > tiles) or -(-tiles // warps) > 16:
                    continue
                out.append({"kind": "tiled", "cpt": cpt, "halo": halo,
                            "pf": pf, "warps": warps, "exchange": exch})
    return out


def tune_march(kernels, cache=True, dtype=torch.float32):
    """Launch shape of the single-instance forward substitution."""
    dev = torch.cuda.get_device_name(kernels.device)
    key = "wave_march4|%s|%s|nx%d|nt%d" % (dev, str(dtype), kernels.nx,
                                           _pow2_bucket(kernels.nt))
    data = _load() if cache else {}
    table = kernels.__dict__.setdefault("march_tune_table", {})
    if key in data:
        table[str(dtype)] = data[key].get("tried")
        return data[key]["cfg"]
    b = torch.zeros(kernels.shape, dtype=dtype, device=kernels.device)
    x = torch.empty_like(b)
    if dtype == torch.float32:
        kernels.initial_rhs(b)
    else:
        b.normal_(generator=torch.Generator(kernels.device).manual_seed(0))
    best = None
    results = []
    for cfg in candidates_march(kernels.nx, dtype):
        try:
            t = _time(lambda: kernels.march_shape(b, x, cfg))
        except OdilError as e:
            if e.status != ODIL_ERR_SHAPE:
                raise
            continue  # e.g. a cluster that does not fit on this device
        results.append((t, cfg))
        if best is None or t < best[0]:
            best = (t, cfg)
    table[str(dtype)] = [[t, c] for t, c in results]
    if cache:
        data[key] = {"cfg": best[1], "ms": best[0],
                     "tried": [[t, c] for t, c in results]}
        _store(data)
    return best[1]
