"""Launch-configuration autotuner.

Results never depend on the tuning -- neighbour sets are fixed by the exact
predicates and every sum has a fixed order -- only the speed does.  The
autotuner times a few complete steps for each candidate (cell width factor of
the fluid/wall grids, threads per block of the fluid loops, porosity
implementation) on a fresh copy of the case, picks the fastest, and caches it
in a small JSON file keyed by the case's sizes and the GPU name.
"""
from __future__ import annotations

import itertools
import json
import os
from pathlib import Path

import torch

# Fluid counts up to which one warp per particle is a candidate (beyond it one
# thread per particle already fills the GPU).
WARP_LANES_MAX_FLUID = 200_000

CACHE = Path(os.environ.get("SPHDEM_AUTOTUNE_CACHE", Path.home() / ".cache" / "warp_sph_gpt_gb300" / "autotune.json"))


def case_key(P, B, D, W, ninst: int = 1) -> str:
    name = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    return f"{name}|fluid={P.n}|wall={B.n}|dem={D.n}|dembnd={W.n}|inst={ninst}"


def candidates(ninst: int = 1, n_fluid: int = 0):
    """Launch options: cell width factor, threads per block, porosity
    implementation (staged only for single-instance grids) and, for systems
    small enough that one thread per particle leaves the GPU idle, one warp
    per particle."""
    variants = (0, 1) if ninst <= 1 else (0,)
    lanes = (1, 32) if 0 < n_fluid <= WARP_LANES_MAX_FLUID else (1,)
    for cf, block, por, ln in itertools.product((1.0, 0.75), (128, 256), variants, lanes):
        yield {"cell_factor": cf, "block_sph": block, "porosity_variant": por, "lanes_sph": ln}


def time_config(make_case, config: dict, warmup: int = 3, steps: int = 8) -> float:
    """ms per step of a fresh case (make_case(cell_factor) -> runner) under config."""
    runner = make_case(config["cell_factor"])
    runner.tune({k: v for k, v in config.items() if k != "cell_factor"})
    runner.run(0, warmup)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record()
    runner.run(warmup, steps)
    end.record()
    torch.cuda.synchronize()
    return start.elapsed_time(end) / steps


def autotune(make_case, key: str, ninst: int = 1, use_cache: bool = True, log=None, timer=time_config,
             cache_path: Path | None = None, n_fluid: int = 0) -> dict:
    """Best configuration for the case behind make_case; cached by key."""
    path = Path(cache_path) if cache_path is not None else CACHE
    cache = {}
    if use_cache and path.exists():
        try:
            cache = json.loads(path.read_text())
        except ValueError:
            cache = {}
    if use_cache and key in cache:
        return cache[key]
    table = []
    for cfg in candidates(ninst, n_fluid):
        ms = timer(make_case, cfg)
        table.append((ms, cfg))
        if log:
            log(f"autotune {cfg}: {ms:.3f} ms/step")
    best = dict(min(table, key=lambda t: t[0])[1])
    best["ms_per_step"] = min(t[0] for t in table)
    cache[key] = best
    if use_cache:
        path.parent.mkdir(parents=True, exist_ok=True)
        path.write_text(json.dumps(cache, indent=1))
    return best
