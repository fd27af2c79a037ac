"""libccc.so (include/ccc.h) against the reference's own ccc_* library:
critical curves, caustics, lens positions, bounding boxes and the
print_ccc file, on triple lenses and on the binary (m3 = 0) path, in the
call order of the reference's scripts (get_cc + get_ca, or get_ca alone)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ccc.npz")
# the reference is built with -Ofast (FMA contraction, reciprocal
# division); the branches agree in order and to FP64 rounding
TOL = 1e-9


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="module")
def ccc_lib(product_lib):
    return os.path.join(os.path.dirname(product_lib), "libccc.so")


def _numbers(text):
    rows = [l for l in text.splitlines() if l and not l.startswith("#")]
    return [[float(x) for x in r.split()] for r in rows]


@pytest.mark.parametrize("k", range(5))
def test_ccc_matches_reference(golden, ccc_lib, k, tmp_path):
    from triplelens_gb300.ccc import CCC
    a, b, th, m2, m3, length = golden["cases"][k]
    length = int(length)
    c = CCC(a, b, th, m2, m3, length, lib_path=ccc_lib)
    if m3 != 0.0:
        c.get_cc()
    c.get_ca()
    order = 4 if m3 == 0.0 else 6
    cc = np.zeros(order * length, np.cdouble)
    ca = np.zeros(order * length, np.cdouble)
    c.copy_cc_ca(cc, ca)
    assert np.max(np.abs(cc - golden["cc_%d" % k])) < TOL
    assert np.max(np.abs(ca - golden["ca_%d" % k])) < TOL
    lz = np.zeros(3, np.cdouble)
    c.copy_lenses(lz)
    assert np.max(np.abs(lz - golden["lenses_%d" % k])) < 1e-15
    box = [np.zeros(1, np.cdouble) for _ in range(4)]
    c.get_bounding_box(*box, 1.1)
    assert np.max(np.abs(np.concatenate(box) - golden["box_%d" % k])) < TOL
    if "text_%d" % k in golden.files:
        f = tmp_path / "ccc.txt"
        c.print_ccc(str(f))
        mine, ref = f.read_text(), str(golden["text_%d" % k])
        assert mine.splitlines()[:2] == ref.splitlines()[:2]
        assert len(mine.splitlines()) == len(ref.splitlines())
        a_, b_ = np.array(_numbers(mine)), np.array(_numbers(ref))
        assert a_.shape == b_.shape
        # values printed with 4 or 6 significant digits: at most one unit in
        # the last printed digit apart (values that are zero to rounding
        # print as arbitrary tiny numbers)
        assert np.all(np.abs(a_ - b_) <= np.maximum(1.01e-3 * np.abs(b_), 1e-12))
