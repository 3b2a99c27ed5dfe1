"""Index arithmetic of the Angles2Coords kernels' aligned span copies (copy_span and
stage_span_async in tpl_a2c.cu), checked on the CPU.

A chunk's n words go between a global span that starts at word offset sh (0..3)
inside its 16-byte block and a 16-byte-aligned staging row where they start at
offset sh too.  The warp walks the 16-byte blocks b = lane, lane + 32, ... of the
global span's aligned cover: a block lying whole inside the span moves as one
vector access (global words base + 4b .. base + 4b + 3 <-> staging words 4b .. 4b + 3),
any other block word by word, only for the words inside the span.  The model below
replays both directions for every phase and length a chunk can have and checks that
every word of the span is moved exactly once with the right value, that nothing
outside the span (or past the staging row's 4 words of slack) is touched, and that
every vector access is 16-byte aligned on both sides.
"""
import pytest

STAGE_WORDS = 32 * 14 * 3 + 4  # coordinate staging row: 32 residues x 14 atoms x 3 floats + slack


def replay(sh, n, lanes=32):
    """Moves of one span: ('vec', global word, staging word) or ('word', global, staging)."""
    moves = []
    nb = (n + sh + 3) >> 2
    for lane in range(lanes):
        for b in range(lane, nb, lanes):
            lo = 4 * b - sh
            if lo >= 0 and lo + 4 <= n:
                moves.append(("vec", sh + lo, 4 * b))  # global word index relative to the aligned base
            else:
                for e in range(4):
                    if 0 <= lo + e < n:
                        moves.append(("word", sh + lo + e, sh + lo + e))
    return moves


@pytest.mark.parametrize("sh", [0, 1, 2, 3])
def test_span_moves_cover_exactly_once(sh):
    for n in list(range(0, 70)) + [3 * 267, 3 * 448, 448, 449, 1343, 1344]:
        seen = {}
        for kind, g, s in replay(sh, n):
            words = range(4) if kind == "vec" else range(1)
            if kind == "vec":
                assert g % 4 == 0 and s % 4 == 0, (sh, n, g, s)  # both sides 16-byte aligned
            for k in words:
                gw, sw = g + k, s + k
                assert sh <= gw < sh + n, (sh, n, gw)  # only words of the span
                assert sw == gw, (sh, n, gw, sw)  # staging keeps the global phase
                assert sw < STAGE_WORDS or n > 3 * 448, (sh, n, sw)
                seen[gw] = seen.get(gw, 0) + 1
        assert sorted(seen) == list(range(sh, sh + n)), (sh, n)
        assert all(c == 1 for c in seen.values()), (sh, n)


def test_staging_row_holds_the_largest_chunk():
    # the largest chunk (32 residues of 14 atoms) at the largest phase fits the row
    assert 3 + 3 * 32 * 14 <= STAGE_WORDS
    assert STAGE_WORDS * 4 % 16 == 0  # rows of a warp stay 16-byte aligned
