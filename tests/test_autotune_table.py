"""The autotuner's shipped table (torchproteinlibrary_gb300/tuned/*.json), which the
Angles2Backbone layer reads through autotune.options_for: every entry names a scheme
and tile the library accepts, and every bucket of the tuning grid is present."""
import glob
import json
import os

import pytest

PKG = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "torchproteinlibrary_gb300")
FWD_OK = {1: (1, 2, 4, 8), 128: (1, 2, 4, 8), 32: (4, 8), 4: (4, 8)}
BWD_OK = {32: (4, 8), 4: (4, 8)}


def tables():
    return sorted(glob.glob(os.path.join(PKG, "tuned", "*.json")))


def test_a_table_ships_for_gb300():
    assert os.path.join(PKG, "tuned", "NVIDIA_GB300.json") in tables()


@pytest.mark.parametrize("path", tables())
def test_table_entries_are_valid_options(path):
    from torchproteinlibrary_gb300 import autotune
    t = json.load(open(path))
    for B in autotune.TABLE_BATCHES:
        for L in autotune.TABLE_LENGTHS:
            assert autotune._bucket(B, L) in t
    for bucket, e in t.items():
        (rpt, cta), (brpt, bufs, bcta) = autotune._entry_options(e)
        assert rpt in FWD_OK[cta], (bucket, rpt, cta)
        assert brpt in BWD_OK[bcta] and bufs in (0, 1, 2) and not (bufs == 2 and brpt == 8), bucket
        assert e["coord_max_A"] <= autotune.COORD_BOUND
