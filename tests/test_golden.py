"""The oracle regenerates the committed golden fixtures (tests/golden/*.npz,
written by tests/golden/make_golden.py): a regression pin of the oracle.
Same machine: bit-identical; the bar is 1e-13 relative so that a host whose
libm rounds a transcendental differently still passes."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="module")
def maker(orc):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.mark.parametrize("name", ["su2_fp64_6cube", "su3_fp64_4x4x6", "cpic_su2_12x6x6", "cgc_su2_20x6x6"])
def test_oracle_reproduces_golden(maker, name):
    ref = load(name)
    got = maker.CASES[name]()
    assert set(got) == set(ref)
    for k in ref:
        a, b = np.asarray(got[k]), ref[k]
        assert a.shape == b.shape, k
        if a.dtype.kind in "iub":
            assert np.array_equal(a, b), k
        else:
            scale = max(float(np.abs(b).max()) if b.size else 0.0, 1e-300)
            assert np.abs(a - b).max() <= 1e-13 * scale, k
