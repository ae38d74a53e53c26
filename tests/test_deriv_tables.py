"""PHOperator / BSOperator construction on the CPU (src/operators/PHOperator.cpp,
BSOperator.cpp): the reference's table files are read in its own format
(PHCalculator.cpp:44-74, BSCalculator.cpp:44-74; the tables here come from the
reference's share/mwfilters, tests/golden/deriv_tables_ref.npz), the operator
equals the one built from the same three matrices directly, and the reader's
errors are the reference's.
"""
import os

import numpy as np
import pytest

import mrcpp_gb300 as mw

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "deriv_tables_ref.npz"))


def write_table_file(path, tables, kp1_last):
    """The reference's layout: for kp1 = 2 .. kp1_last a line with kp1 and
    3 kp1 rows of kp1 numbers (rows of orders without a fixture are zero)."""
    with open(path, "w") as fh:
        for kp1 in range(2, kp1_last + 1):
            fh.write("%d\n" % kp1)
            data = tables.get(kp1, np.zeros((3 * kp1, kp1)))
            for row in data:
                fh.write(" ".join("%.17e" % v for v in row) + " \n")


def filter_dir(tmp_path, t, kind, n, k):
    name = ("%s_ph_deriv_%d.txt" if kind == "ph" else "%s_b-spline-deriv%d.txt") % (t, n)
    write_table_file(tmp_path / name, {k + 1: GOLDEN["%s_%s%d_%d" % (t, kind, n, k)]}, k + 1)
    return str(tmp_path)


@pytest.mark.parametrize("kind,n", [("ph", 1), ("ph", 2), ("bs", 1), ("bs", 2), ("bs", 3)])
@pytest.mark.parametrize("basis,t,k", [(mw.LEGENDRE, "L", 7), (mw.INTERPOLATING, "I", 5)])
def test_table_operator_from_files(tmp_path, kind, n, basis, t, k):
    mra = mw.MRA(box=(-20, 20), order=k, basis=basis)
    d = filter_dir(tmp_path, t, kind, n, k)
    cls = mw.PHOperator if kind == "ph" else mw.BSOperator
    D = cls(mra, n, d)
    K = k + 1
    S = GOLDEN["%s_%s%d_%d" % (t, kind, n, k)]
    E = mw.TableDerivativeOperator(mra, n, S[:K], S[K:2 * K], S[2 * K:])
    a, b = D.export(), E.export()
    assert D.n_terms == 1 and D.n_nodes == E.n_nodes
    for key in ("depth", "max_transl", "blocks", "norms"):
        assert np.array_equal(a[key], b[key]), key
    # the band: translations -1, 0, 1 at every depth, nonzero blocks
    assert a["max_transl"].max() >= 1
    assert np.abs(a["blocks"]).max() > 0
    # MWFILTERS_DIR is used when no directory is given
    os.environ["MWFILTERS_DIR"] = d
    try:
        F = cls(mra, n)
    finally:
        os.environ.pop("MWFILTERS_DIR", None)
    assert np.array_equal(F.export()["blocks"], a["blocks"])


def test_table_operator_errors(tmp_path):
    mra = mw.MRA(box=(-20, 20), order=5, basis=mw.LEGENDRE)
    with pytest.raises(RuntimeError, match="order"):
        mw.PHOperator(mra, 3, str(tmp_path))
    with pytest.raises(RuntimeError, match="order"):
        mw.BSOperator(mra, 4, str(tmp_path))
    with pytest.raises(RuntimeError, match="Failed to open"):
        mw.PHOperator(mra, 1, str(tmp_path))
    os.environ.pop("MWFILTERS_DIR", None)
    with pytest.raises(RuntimeError, match="filter directory"):
        mw.BSOperator(mra, 1)
    # a file whose order lines do not count up
    (tmp_path / "L_ph_deriv_1.txt").write_text("3\n")
    with pytest.raises(RuntimeError, match="Orders do not match"):
        mw.PHOperator(mra, 1, str(tmp_path))
    # orders beyond the file's last table
    write_table_file(tmp_path / "L_b-spline-deriv1.txt", {}, 4)
    with pytest.raises(RuntimeError):
        mw.BSOperator(mra, 1, str(tmp_path))
