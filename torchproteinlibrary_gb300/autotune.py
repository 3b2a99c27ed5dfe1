"""Autotuner for the Angles2Backbone FP32 kernels.

Knobs (tpl_options): residues per thread R (the scan tile is 32 R residues for
warp tiles, 128 R for CTA tiles, a 32 R-residue chunk for one warp per chain),
the scan scheme (warp tiles, CTA tiles, one warp or one CTA per chain), the length from
which inter-tile carries are composed in FP64, and the residues per lane of the
backward from coordinates.  For a shape
(batch, max_len) the tuner times forward+backward of every candidate on
synthetic chains of that shape with CUDA events and keeps the fastest whose
coordinates stay within the accuracy bound of the FP64 form.  Results are
cached per GPU name and shape bucket in a JSON file
($TPL_TUNE_CACHE, default ~/.cache/torchproteinlibrary_gb300/tune.json).
"""
from __future__ import annotations

import json
import math
import os

import torch

from . import load_extension

CANDIDATES = [
    # (residues_per_thread, threads_per_cta)  threads_per_cta 1 = warp tiles, 128 = CTA tiles
    (1, 1), (2, 1), (4, 1), (8, 1), (2, 128), (4, 128), (8, 128),
    # threads_per_cta 32 = one warp per chain, chunks of 32 R residues; 4 = one CTA of four warps
    # per chain, chunks dealt round the warps
    (4, 32), (8, 32), (4, 4), (8, 4),
]
COORD_BOUND = 1e-3  # A, against the FP64 form


def _cache_path() -> str:
    return os.environ.get("TPL_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "torchproteinlibrary_gb300", "tune.json"))


def _bucket(batch: int, max_len: int) -> str:
    b = 1 << max(0, math.ceil(math.log2(max(1, batch))))
    l = 128 * max(1, math.ceil(max_len / 128))
    return f"{b}x{l}"


def _load_cache() -> dict:
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except Exception:
        return {}


def _save_cache(d: dict) -> None:
    p = _cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
    except OSError:
        pass


def _time_options(rm, opts, ang, lengths, up, steps):
    """Mean forward and backward milliseconds for one option set (CUDA events)."""
    rm.set_options(*opts)
    B, _, L = ang.shape
    ws = torch.zeros(rm.workspace_bytes(B, L), dtype=torch.uint8, device=ang.device)
    coords = torch.empty(B, 9 * L, device=ang.device)
    gang = torch.empty(B, 3, L, device=ang.device)
    none = torch.empty(0, device=ang.device)
    for _ in range(2):
        rm.Angles2BackboneGPU_forward(ang, coords, lengths, ws)
        rm.Angles2BackboneGPU_backward(gang, up, ang, lengths, ws, none)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    e[0].record()
    for _ in range(steps):
        rm.Angles2BackboneGPU_forward(ang, coords, lengths, ws)
    e[1].record()
    for _ in range(steps):
        rm.Angles2BackboneGPU_backward(gang, up, ang, lengths, ws, none)
    e[2].record()
    torch.cuda.synchronize(ang.device)
    return e[0].elapsed_time(e[1]) / steps, e[1].elapsed_time(e[2]) / steps, coords, gang


def _errors(rm, ang, lengths, up, coords, gang, n=64):
    n = min(n, ang.shape[0])
    a64 = ang[:n].double().contiguous()
    L = ang.shape[2]
    c64 = torch.empty(n, 9 * L, dtype=torch.float64, device=ang.device)
    g64 = torch.empty(n, 3, L, dtype=torch.float64, device=ang.device)
    ws = torch.zeros(rm.workspace_bytes(n, L), dtype=torch.uint8, device=ang.device)
    rm.Angles2BackboneGPU_forward(a64, c64, lengths[:n].contiguous(), ws)
    rm.Angles2BackboneGPU_backward(g64, up[:n].double().contiguous(), a64, lengths[:n].contiguous(), ws,
                                   torch.empty(0, device=ang.device))
    d = (coords[:n].double() - c64).view(n, -1, 3).norm(dim=-1)
    return float(d.max()), float(d.pow(2).mean().sqrt()), float((gang[:n].double() - g64).abs().max() / g64.abs().max())


def sweep(ang, lengths, up, candidates=CANDIDATES, carry_thresholds=(0,), steps=5):
    """Time every (candidate, carry threshold) on these inputs; returns a list of dicts."""
    rm = load_extension("_ReducedModel")
    saved = rm.get_options()
    out = []
    try:
        for r, cta in candidates:
            for thr in carry_thresholds:
                opts = (r, thr, 0, 0, cta)
                f, b, coords, gang = _time_options(rm, opts, ang, lengths, up, steps)
                cmax, crms, grel = _errors(rm, ang, lengths, up, coords, gang)
                out.append({"residues_per_thread": r, "threads_per_cta": cta, "fp64_carry_min_len": thr,
                            "fwd_ms": f, "bwd_ms": b, "coord_max_A": cmax, "coord_rms_A": crms, "grad_max_rel": grel})
    finally:
        rm.set_options(*saved)
    return out


# backward from coordinates: (residues per lane, chunk buffers, scheme: 32 = one warp per chain,
# 4 = one CTA of four warps per chain)
COORDS_BWD_CANDIDATES = ((4, 1, 32), (4, 2, 32), (8, 1, 32), (4, 1, 4), (4, 2, 4), (8, 1, 4))


def sweep_backward_coords(ang, lengths, up, candidates=COORDS_BWD_CANDIDATES, steps=5):
    """Time the float32 backward from the forward's coordinates for each residues-per-lane
    value (the forward runs once with the current options); returns a list of dicts
    with the gradient error against the FP64 form."""
    rm = load_extension("_ReducedModel")
    saved = tuple(rm.get_backward_options())
    B, _, L = ang.shape
    ws = torch.zeros(rm.workspace_bytes(B, L), dtype=torch.uint8, device=ang.device)
    coords = torch.empty(B, 9 * L, device=ang.device)
    rm.Angles2BackboneGPU_forward(ang, coords, lengths, ws)
    gang = torch.empty(B, 3, L, device=ang.device)
    out = []
    try:
        for c, nb, sch in candidates:
            rm.set_backward_options(c, nb, sch)
            for _ in range(2):
                rm.Angles2BackboneGPU_backward_coords(gang, up, coords, lengths, ws)
            e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            e[0].record()
            for _ in range(steps):
                rm.Angles2BackboneGPU_backward_coords(gang, up, coords, lengths, ws)
            e[1].record()
            torch.cuda.synchronize(ang.device)
            _, _, grel = _errors(rm, ang, lengths, up, coords, gang)
            out.append({"residues_per_thread": c, "copy_buffers": nb, "threads_per_cta": sch,
                        "bwd_ms": e[0].elapsed_time(e[1]) / steps, "grad_max_rel": grel})
    finally:
        rm.set_backward_options(*saved)
    return out


def tune(ang, lengths, up, use_cache=True, steps=5):
    """Pick and install, for this shape, the fastest forward candidate whose
    coordinates stay within COORD_BOUND, and the fastest backward from coordinates
    (what the float32 layer runs).  The returned dict describes the forward choice
    and carries the backward's under "backward_coords"."""
    rm = load_extension("_ReducedModel")
    key = f"{torch.cuda.get_device_name(ang.device)}|{_bucket(ang.shape[0], ang.shape[2])}|v2"
    cache = _load_cache() if use_cache else {}
    rows, brows = [], []
    if key in cache and "backward_coords" in cache[key]:
        best = cache[key]
    else:
        rows = sweep(ang, lengths, up, steps=steps)
        ok = [r for r in rows if r["coord_max_A"] <= COORD_BOUND] or rows
        best = dict(min(ok, key=lambda r: r["fwd_ms"]))
        rm.set_options(best["residues_per_thread"], best["fp64_carry_min_len"], 0, 0, best["threads_per_cta"])
        brows = sweep_backward_coords(ang, lengths, up, steps=steps)
        best["backward_coords"] = min(brows, key=lambda r: r["bwd_ms"])
        cache[key] = best
        if use_cache:
            _save_cache(cache)
    rm.set_options(best["residues_per_thread"], best["fp64_carry_min_len"], 0, 0, best["threads_per_cta"])
    bc = best["backward_coords"]
    rm.set_backward_options(bc["residues_per_thread"], bc.get("copy_buffers", 0), bc.get("threads_per_cta", 0))
    tune.last_sweep = rows
    tune.last_backward_sweep = brows
    return best
