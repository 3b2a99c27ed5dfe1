"""Pin the oracle's numpy restatements of CoordsTransform, Coords2TypedCoords and
Coords2RMSD to the reference itself.

The fixtures tests/golden/{transform,typed,rmsd}_ref.npz were written by
tests/golden/make_golden.py, which runs the reference's own Python layers over its
own CPU interfaces (coordsTransform_interface.cpp, coords2typedcoords_interface.cpp,
coords2rmsd_interface.cpp, compiled unmodified by oracle/build_ref_ext.py).  If a
restatement drifts from the reference, these tests fail.

Tolerances: translate, centre, bounding box, typed coordinates and their backwards
are single copies or the same additions in the same order (exact); rotate 1e-14 of
the coordinate scale in FP64 (different FMA contraction) and 1 FP32 ulp of it in
FP32; Coords2RMSD 1e-10 relative (the reference solves the 4x4 eigenproblem with
torch, the oracle with numpy).
"""
import os

import numpy as np

import oracle

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLD, name))


def test_rotation_from_u_matches_reference():
    d = _load("transform_ref.npz")
    np.testing.assert_array_equal(oracle.rotation_from_u(d["u"]), d["rotation"])


def test_transform_matches_reference():
    d = _load("transform_ref.npz")
    na = d["num_atoms"]
    for tag, rot_tol in (("f64", 1e-14), ("f32", 2.0 ** -23)):
        x = d[f"{tag}_x"]
        scale = np.abs(x).max()
        R = d["rotation"].astype(x.dtype)
        np.testing.assert_array_equal(oracle.coords_translate(x, d[f"{tag}_T"], na), d[f"{tag}_translate"])
        np.testing.assert_array_equal(oracle.coords_translate(d[f"{tag}_grad_out"], None, na),
                                      d[f"{tag}_translate_grad"])
        assert np.abs(oracle.coords_rotate(x, R, na) - d[f"{tag}_rotate"]).max() <= rot_tol * scale
        g = d[f"{tag}_grad_out"]
        assert np.abs(oracle.coords_rotate(g, R, na, transpose=True) - d[f"{tag}_rotate_grad"]).max() <= \
            rot_tol * np.abs(g).max() * 4
        np.testing.assert_array_equal(oracle.coords_center_backward(d[f"{tag}_grad_center"], na, x.shape[1] // 3),
                                      d[f"{tag}_center_grad"])
        lo, hi = oracle.coords_bbox(x, na)
        np.testing.assert_array_equal(lo, d[f"{tag}_bbox_lo"])
        np.testing.assert_array_equal(hi, d[f"{tag}_bbox_hi"])
    # the reference sums the centre serially in the coordinate type; the oracle in FP64
    np.testing.assert_array_equal(oracle.coords_center(d["f64_x"], na), d["f64_center"])
    c32 = oracle.coords_center(d["f32_x"], na)
    assert np.abs(c32 - d["f32_center"]).max() <= 8 * 2.0 ** -23 * np.abs(d["f32_x"]).max()


def test_typed_coords_match_reference():
    d = _load("typed_ref.npz")
    typed, counts, offsets, index = oracle.typed_coords(d["coords"], d["res_names"], d["atom_names"], d["num_atoms"])
    np.testing.assert_array_equal(counts, d["num_atoms_of_type"])
    np.testing.assert_array_equal(offsets, d["offsets"])
    np.testing.assert_array_equal(typed, d["typed"])
    grad = oracle.typed_coords_backward(d["grad_typed"], counts, index, d["coords"].shape[1] // 3)
    np.testing.assert_array_equal(grad, d["grad_coords"])


def test_rmsd_matches_reference():
    d = _load("rmsd_ref.npz")
    rmsd, UT, gfac = oracle.rmsd(d["src"], d["dst"], d["num_atoms"])
    np.testing.assert_allclose(rmsd, d["rmsd"], rtol=1e-10, atol=0)
    np.testing.assert_allclose(UT, d["ut"], rtol=0, atol=1e-10)
    grad = gfac * d["grad_rmsd"][:, None]
    assert np.abs(grad - d["grad_src"]).max() <= 1e-10 * np.abs(d["grad_src"]).max()
    # two of the pairs are rigidly moved noisy copies: small but non-zero RMSD
    assert d["rmsd"][2] < 0.5 and d["rmsd"][3] < 0.5
