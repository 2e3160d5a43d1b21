"""Launch-configuration autotuner of the burn.

The sparse and mixed solvers run in one of two warp-cooperative particle layouts (one warp
per particle, or 32 particles per warp in lockstep), and the batched layout takes the number
of particles in flight per warp (1..32).  Which is fastest depends on the network, the EOS,
the batch size and how uneven the particles' Newton-iteration counts are, so the choice is
measured: every candidate burns a copy of (a sample of) the caller's particles on the
device, timed with CUDA events, and the fastest is cached per (device, network, EOS, solver,
batch-size class) in a JSON file and applied to the context.  All candidates compute the
same per-particle results (the parity tests hold for every layout)."""
import json
import math
import os

CANDIDATES = [("batched", 32), ("batched", 16), ("batched", 8), ("batched", 4), ("warp", 32)]
CACHE_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_autotune_cache.json")


def size_class(P):
    """Batch-size class: floor(log2(P)), so that batches within a factor 2 share a choice."""
    return int(math.floor(math.log2(max(int(P), 1))))


def cache_key(device_name, network, eos, solver, P):
    return f"{device_name}|net{int(network)}|eos{int(eos)}|solver{int(solver)}|p2^{size_class(P)}"


def load_cache(path=CACHE_PATH):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def store_cache(cache, path=CACHE_PATH):
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def apply(ctx, choice):
    """Set the context's layout and slots per warp from a choice dict."""
    ctx.set_layout(choice["layout"])
    ctx.set_batch_slots(choice["slots"])


def tune(ctx, network, Y, T, rho, dt, hydro_dt, eos, mu=0.0, solver=1, max_iter=100000, sample=65536,
         candidates=CANDIDATES, cache_path=CACHE_PATH, use_cache=True):
    """Choose and apply the fastest launch configuration for burning these particles.

    Y is a [species, particles] float64 CUDA tensor (or a list of rows); T, rho, dt 1-D CUDA
    tensors.  At most `sample` particles (taken evenly over the batch) are burned per
    candidate, on copies: the caller's arrays are not modified.  Returns the choice dict
    {"layout", "slots", "ms", "timings"}."""
    import torch
    import nnet_gb300 as nn
    rows = torch.stack([Y[j] for j in range(network)]) if isinstance(Y, (list, tuple)) else Y
    P = T.numel()
    dev = T.device
    key = cache_key(torch.cuda.get_device_name(dev), network, eos, solver, P)
    cache = load_cache(cache_path) if use_cache else {}
    if key in cache:
        apply(ctx, cache[key])
        return cache[key]
    idx = torch.linspace(0, P - 1, steps=min(P, sample), device=dev).round().long().unique()
    Y0, T0, rho0, dt0 = rows[:, idx].contiguous(), T[idx].contiguous(), rho[idx].contiguous(), dt[idx].contiguous()
    timings = {}
    for layout, slots in candidates:
        ctx.set_layout(layout)
        ctx.set_batch_slots(slots)
        Yc, Tc, dtc = Y0.clone(), T0.clone(), dt0.clone()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ctx.burn(network, Yc, Tc, rho0, dtc, hydro_dt, eos=eos, mu=mu, solver=solver, max_iter=max_iter)
        e1.record()
        torch.cuda.synchronize(dev)
        timings[f"{layout}/{slots}"] = e0.elapsed_time(e1)
    best = min(timings, key=timings.get)
    layout, slots = best.split("/")
    choice = {"layout": layout, "slots": int(slots), "ms": timings[best], "timings": timings,
              "sample": int(idx.numel())}
    apply(ctx, choice)
    if use_cache:
        cache[key] = choice
        store_cache(cache, cache_path)
    return choice
