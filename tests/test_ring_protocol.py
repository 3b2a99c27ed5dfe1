"""Handoff schedule of the kernels that share a chain between the W warps of a CTA
(a2b_fwd_ring_kernel, a2b_bwd_coords_ring_kernel with W = 4; a2c_fwd_ring_kernel,
a2c_bwd_coords_ring_kernel with W = 4 or 8), checked on the CPU before any GPU runs
it.

Each warp of the CTA owns the chunks the kernels give it (forward: chunk k on warp
k % W, visited in ascending order; backward: chunk k on warp (nchunk - 1 - k) % W,
visited in descending order).  The carry into chunk k passes under named barrier
1 + k % W with 64 threads: the producer warp arrives (bar.arrive), the consumer warp
syncs (bar.sync).  The model below replays every warp's sequence of barrier
operations under random interleavings, with the hardware rule that a barrier phase
completes once 64 threads (two warps) have arrived.  It checks that no schedule
deadlocks and that every phase joins exactly the producer and the consumer of one
handoff (a barrier id is never shared by two handoffs in flight).
"""
import random

import pytest

def warp_programs(nchunk, forward, WARPS):
    progs = {w: [] for w in range(WARPS)}
    for w in range(WARPS):
        if forward:
            for k in range(w, nchunk, WARPS):
                if k > 0:
                    progs[w].append(("sync", k))
                if k + 1 < nchunk:
                    progs[w].append(("arrive", k + 1))
        else:
            k = nchunk - 1 - w
            while k >= 0:
                assert (nchunk - 1 - k) % WARPS == w
                if k + 1 < nchunk:
                    progs[w].append(("sync", k))
                if k > 0:
                    progs[w].append(("arrive", k - 1))
                k -= WARPS
    return progs


def replay(progs, rng, WARPS):
    pc = {w: 0 for w in progs}
    blocked = set()
    phase = {}
    while True:
        ready = [w for w in progs if pc[w] < len(progs[w]) and w not in blocked]
        if not ready:
            return ("deadlock", sorted(blocked)) if blocked else ("ok", None)
        w = rng.choice(ready)
        op, k = progs[w][pc[w]]
        pc[w] += 1
        bid = 1 + k % WARPS
        members = phase.setdefault(bid, [])
        members.append((w, op, k))
        if op == "sync":
            blocked.add(w)
        if len(members) == 2:
            if len({m[2] for m in members}) != 1 or sorted(m[1] for m in members) != ["arrive", "sync"]:
                return "mixed", members
            for m in members:  # the phase releases its syncing warp; the arriving one never waited here
                if m[1] == "sync":
                    blocked.discard(m[0])
            phase[bid] = []


@pytest.mark.parametrize("warps", [4, 8])
@pytest.mark.parametrize("forward", [True, False])
def test_ring_handoffs_never_deadlock_or_mix(forward, warps):
    for nchunk in range(0, 40):
        progs = warp_programs(nchunk, forward, warps)
        n_sync = sum(op == "sync" for p in progs.values() for op, _ in p)
        n_arrive = sum(op == "arrive" for p in progs.values() for op, _ in p)
        assert n_sync == n_arrive == max(0, nchunk - 1)
        for seed in range(200):
            result, info = replay(progs, random.Random(seed), warps)
            assert result == "ok", (nchunk, seed, result, info)
