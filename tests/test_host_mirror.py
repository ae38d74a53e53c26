"""Host mirror of MRCPP's data model (CPU): world boxes, projection, norms,
transforms, copy_grid, dot, flat export/import."""
import math

import numpy as np
import pytest

import mrcpp_gb300 as mw
from cases import gaussian_sum, project, unit_gaussian


@pytest.mark.parametrize("box,scale,sf", [((-20, 20), -4, 1.25), ((-32, 32), -5, 1.0), ((0, 1), 0, 1.0)])
def test_world_box(box, scale, sf):
    # BoundingBox({lb, ub}) halves the box until the unit length is below 2 (BoundingBox.cpp:47-80)
    mra = mw.MRA(box=box, order=3)
    assert mra.root_scale == scale
    assert mra.sf == pytest.approx(sf)
    assert mra.max_scale == scale + 30


@pytest.mark.parametrize("basis,order", [(mw.INTERPOLATING, 5), (mw.LEGENDRE, 7)])
def test_projection_norm_and_integral(basis, order):
    mra = mw.MRA(box=(-20, 20), order=order, basis=basis)
    beta = 10.0
    f = project(mra, 1e-5, unit_gaussian(beta, (0.1, 0.2, -0.3)))
    assert f.integrate() == pytest.approx(1.0, abs=1e-6)
    exact = (beta / math.pi) ** 3 * (math.pi / (2 * beta)) ** 1.5
    assert f.square_norm == pytest.approx(exact, rel=1e-8)
    assert math.sqrt(mw.dot(f, f)) == pytest.approx(math.sqrt(exact), rel=1e-8)
    assert f.evalf((0.1, 0.2, -0.3)) == pytest.approx((beta / math.pi) ** 1.5, rel=1e-4)


def test_export_import_roundtrip_and_norms():
    mra = mw.MRA(box=(-32, 32), order=4, basis=mw.LEGENDRE)
    f = project(mra, 1e-4, gaussian_sum(3, 3, (1.0, 20.0), (-2.0, 2.0)))
    x = f.export()
    # component norms are the L2 norms of the 8 coefficient blocks
    K3 = mra.kp1 ** 3
    blocks = x["coefs"].reshape(len(x["child0"]), 8, K3)
    np.testing.assert_allclose(x["norms"], np.sqrt((blocks ** 2).sum(-1)), rtol=1e-13)
    g = mw.FunctionTree(mra)
    g.load_flat(x["idx"], x["child0"], x["coefs"], f.square_norm)
    y = g.export()
    np.testing.assert_array_equal(x["idx"], y["idx"])
    np.testing.assert_array_equal(x["child0"], y["child0"])
    np.testing.assert_array_equal(x["coefs"], y["coefs"])
    assert mw.dot(f, g) == pytest.approx(f.square_norm, rel=1e-12)


def test_copy_grid_has_topology_and_no_coefficients():
    mra = mw.MRA(box=(-20, 20), order=3, basis=mw.INTERPOLATING)
    f = project(mra, 1e-3, unit_gaussian(20.0, (0, 0, 0)))
    g = mw.FunctionTree(mra)
    mw.copy_grid(g, f)
    a, b = f.export(), g.export()
    np.testing.assert_array_equal(a["idx"], b["idx"])
    np.testing.assert_array_equal(a["child0"], b["child0"])
    assert not b["coefs"].any()
    assert g.square_norm == -1.0


def test_compressed_form_is_consistent():
    # BottomUp after projection: every branch node is the compression of its
    # children, so the scaling part of the parents reproduces the integral
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    f = project(mra, 1e-4, gaussian_sum(9, 2, (2.0, 30.0), (-1.0, 1.0)))
    x = f.export()
    n = len(x["child0"])
    K3 = mra.kp1 ** 3
    tot = 0.0
    for i in range(n):
        if x["child0"][i] < 0:
            tot += (x["norms"][i] ** 2).sum()
    assert tot == pytest.approx(f.square_norm, rel=1e-12)


def test_tree_file_roundtrip(tmp_path):
    # saveTree / loadTree (FunctionTree.cpp:378-435) in the flat tree-file layout:
    # same topology, bit-identical coefficients, square norm and values
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    f = project(mra, 1e-4, gaussian_sum(7, 4, (1.0, 40.0), (-2.0, 2.0)))
    path = str(tmp_path / "density")
    f.saveTree(path)
    assert (tmp_path / "density.mwtree").exists()
    g = mw.FunctionTree(mra)
    g.loadTree(path)
    a, b = f.export(), g.export()
    assert np.array_equal(a["idx"], b["idx"]) and np.array_equal(a["child0"], b["child0"])
    assert np.array_equal(a["coefs"], b["coefs"])
    assert g.square_norm == f.square_norm
    for r in [(0.1, -0.4, 0.3), (1.5, 0.2, -1.0)]:
        assert g.evalf(r) == f.evalf(r)


def test_tree_file_errors(tmp_path):
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.INTERPOLATING)
    f = project(mra, 1e-3, unit_gaussian(5.0, (0.0, 0.0, 0.0)))
    path = str(tmp_path / "f")
    f.saveTree(path)
    # another MRA (order, basis or world) is refused, like loadTree's requirement
    for other in (mw.MRA(box=(-20, 20), order=6, basis=mw.INTERPOLATING), mw.MRA(box=(-20, 20), order=5, basis=mw.LEGENDRE),
                  mw.MRA(box=(-32, 32), order=5, basis=mw.INTERPOLATING)):
        with pytest.raises(mw.MWGPUError):
            mw.FunctionTree(other).loadTree(path)
    # missing, foreign and truncated files
    with pytest.raises(mw.MWGPUError):
        mw.FunctionTree(mra).loadTree(str(tmp_path / "missing"))
    (tmp_path / "junk.mwtree").write_bytes(b"not a tree file at all")
    with pytest.raises(mw.MWGPUError):
        mw.FunctionTree(mra).loadTree(str(tmp_path / "junk"))
    data = (tmp_path / "f.mwtree").read_bytes()
    (tmp_path / "cut.mwtree").write_bytes(data[: len(data) // 2])
    with pytest.raises(mw.MWGPUError):
        mw.FunctionTree(mra).loadTree(str(tmp_path / "cut"))
    # a tree that failed to load keeps its nodes
    h = project(mra, 1e-3, unit_gaussian(5.0, (0.0, 0.0, 0.0)))
    n0 = h.n_nodes
    with pytest.raises(mw.MWGPUError):
        h.loadTree(str(tmp_path / "cut"))
    assert h.n_nodes == n0
