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


def candidates_march(nx):
    out = []
    for cpt in (1, 2, 4, 8):
        threads = ((nx + cpt - 1) // cpt + 31) // 32 * 32
        if cpt > 1 and (nx + cpt - 1) // cpt < 32:
            continue
        for pf in (8, 16):
            if threads <= march_max_threads(cpt, pf):
                out.append({"cpt": cpt, "pf": pf})
    return out


def tune_march(kernels, cache=True):
    """Launch shape of the single-instance FP32 forward substitution."""
    dev = torch.cuda.get_device_name(kernels.device)
    key = "wave_march|%s|nx%d|nt%d" % (dev, kernels.nx,
                                        _pow2_bucket(kernels.nt))
    data = _load() if cache else {}
    if key in data:
        kernels.march_tune_table = data[key].get("tried")
        return data[key]["cfg"]
    b = torch.zeros(kernels.shape, dtype=torch.float32, device=kernels.device)
    x = torch.empty_like(b)
    kernels.initial_rhs(b)
    best = None
    results = []
    for cfg in candidates_march(kernels.nx):
        t = _time(lambda: kernels.march_shape(b, x, cfg["cpt"], cfg["pf"]))
        results.append((t, cfg))
        if best is None or t < best[0]:
            best = (t, cfg)
    kernels.march_tune_table = [[t, c] for t, c in results]
    if cache:
        data[key] = {"cfg": best[1], "ms": best[0],
                     "tried": [[t, c] for t, c in results]}
        _store(data)
    return best[1]
