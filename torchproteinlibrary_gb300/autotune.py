"""Autotuner for the Angles2Backbone FP32 kernels, and the lookup the layer uses.

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

The layer (``ReducedModel.Angles2Backbone``) asks ``options_for`` for every float32
batch: the user's cache first, then the table shipped with the package for this GPU
(``tuned/<gpu name>.json``, written by ``build_table`` on that GPU), and when
neither has the shape's bucket, the library's built-in rule (tpl_options left at 0).
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


# ------------------------------------------------------------ the layer's lookup
_TABLE_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned")
_LOOKUP: dict = {}
_TABLES: dict = {}


def table_file(gpu_name: str) -> str:
    """Path of the shipped table for a GPU name."""
    return os.path.join(_TABLE_DIR, "".join(c if c.isalnum() else "_" for c in gpu_name) + ".json")


def _shipped_table(gpu_name: str) -> dict:
    if gpu_name not in _TABLES:
        try:
            with open(table_file(gpu_name)) as f:
                _TABLES[gpu_name] = json.load(f)
        except (OSError, ValueError):
            _TABLES[gpu_name] = {}
    return _TABLES[gpu_name]


def _entry_options(entry: dict):
    bc = entry["backward_coords"]
    return ((int(entry["residues_per_thread"]), int(entry["threads_per_cta"])),
            (int(bc["residues_per_thread"]), int(bc.get("copy_buffers", 0)), int(bc.get("threads_per_cta", 0))))


def options_for(device, batch: int, max_len: int):
    """((residues_per_thread, threads_per_cta) of the forward, (residues_per_thread,
    copy_buffers, threads_per_cta) of the backward from coordinates) tuned for this
    shape's bucket on this GPU, or None (the library's built-in rule then applies).
    Looked up once per (device, batch, max_len) in the process."""
    key = (device.index, int(batch), int(max_len))
    hit = _LOOKUP.get(key, False)
    if hit is not False:
        return hit
    name = torch.cuda.get_device_name(device)
    bucket = _bucket(batch, max_len)
    entry = _load_cache().get(f"{name}|{bucket}|v2") or _shipped_table(name).get(bucket)
    res = None
    if entry and "backward_coords" in entry:
        try:
            res = _entry_options(entry)
        except (KeyError, TypeError, ValueError):
            res = None
    _LOOKUP[key] = res
    return res


def clear_lookup() -> None:
    """Forget the options looked up so far (after the cache or a table changed)."""
    _LOOKUP.clear()
    _TABLES.clear()


TABLE_BATCHES = (32, 128, 512, 1024, 2048, 4096, 16384)
TABLE_LENGTHS = (64, 128, 256, 384, 512, 768, 1024)


def build_table(device=None, batches=TABLE_BATCHES, lengths=TABLE_LENGTHS, steps=5, seed=0) -> dict:
    """Tune every (batch, max_len) bucket of the grid on this GPU and return the table
    (bucket -> tuned entry) that ``options_for`` reads.  Each bucket is tuned on
    synthetic chains at the bucket's upper shape: lengths uniform on [max_len / 4,
    max_len], phi and psi uniform on [-pi, pi), omega = pi, an N(0, 1) upstream
    gradient.

        python -c "from torchproteinlibrary_gb300 import autotune as t; t.write_table()"
    """
    device = torch.device("cuda") if device is None else device
    g = torch.Generator(device=device).manual_seed(seed)
    table = {}
    for B in batches:
        for L in lengths:
            ang = (torch.rand(B, 3, L, device=device, generator=g) * 2 - 1) * math.pi
            ang[:, 2] = math.pi
            lens = torch.randint(max(1, L // 4), L + 1, (B,), device=device, generator=g, dtype=torch.int32)
            up = torch.randn(B, 9 * L, device=device, generator=g)
            best = dict(tune(ang, lens, up, use_cache=False, steps=steps))
            best["tuned_on"] = f"{B}x{L}, lengths U[{max(1, L // 4)}, {L}]"
            table[_bucket(B, L)] = best
    return table


def write_table(path=None, **kw) -> str:
    """build_table on the current GPU, written where options_for looks for it (or to path)."""
    table = build_table(**kw)
    path = path or table_file(torch.cuda.get_device_name(torch.device("cuda")))
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    return path