"""The SU(3) FP32 leapfrog in plaquette form streamed along dimension 0
(su3_stream.cuh, selected by OPX_STREAM_FP32=1) against the paired staple form
(the default) and the FP64 run on the same initial state.

Both FP32 forms compute FastTYMSolver.CombinedUpdate (FastTYMSolver.java:40-63)
with the staple sum of Grid.getStapleSum (Grid.java:675-696); the plaquette form
regroups the same terms, so the two agree to FP32 rounding: links and E within
2e-5 per link after 20 steps, both within 1e-4 of FP64.  Lattices cover the
periodic wrap of a tile onto itself (N1 = 8, N2 = 32), a single x0 plane,
uneven spacings, and block counts that make each block walk ranges across tile
boundaries (OPX_STREAM_BLOCKS)."""
import os

import numpy as np
import pytest

from helpers import fresh, oracle_ic, link_rel_err, field_rel_err
from openpixi_gb300 import _native as N
from test_gpu_parity import handle_from_oracle, bulk_vec

pytestmark = pytest.mark.gpu


def _handle(g, env, **kw):
    for k, v in env.items():
        os.environ[k] = v
    try:
        return handle_from_oracle(g, **kw)
    finally:
        for k in env:
            os.environ.pop(k, None)


CASES = [
    ((8, 8, 32), (1.0, 1.0, 1.0), None),
    ((1, 8, 32), (1.0, 1.0, 1.0), None),
    ((6, 16, 64), (1.0, 0.9, 1.2), None),
    ((6, 16, 64), (1.0, 1.0, 1.0), "5"),
    ((9, 24, 32), (1.1, 1.0, 0.8), "4"),
    ((32, 32, 32), (1.0, 1.0, 1.0), None),
]


@pytest.mark.parametrize("dims,a,blocks", CASES)
def test_stream_matches_staple_form(native, orc, dims, a, blocks):
    g = fresh(oracle_ic(3, dims, 11, 0.2, 0.2, a=a))
    env = {"OPX_STREAM_FP32": "1"}
    if blocks is not None:
        env["OPX_STREAM_BLOCKS"] = blocks
    hs = _handle(g, env, precision=N.OPX_F32, reunit_every=7)
    hp = _handle(g, {}, precision=N.OPX_F32, reunit_every=7)
    h64 = handle_from_oracle(g)
    for h in (hs, hp, h64):
        h.initialize()
        h.step(20)
    us, up, u64 = (h.download(N.FIELD_U) for h in (hs, hp, h64))
    es, ep, e64 = (h.download(N.FIELD_E) for h in (hs, hp, h64))
    un_s, un_p = hs.download(N.FIELD_UNEXT), hp.download(N.FIELD_UNEXT)
    assert link_rel_err(us, up) <= 2e-5
    assert link_rel_err(un_s, un_p) <= 2e-5
    assert field_rel_err(es, ep) <= 2e-5
    assert link_rel_err(us, u64) <= 1e-4
    assert field_rel_err(es, e64) <= 1e-4
    bs, bp = bulk_vec(hs.reduce()), bulk_vec(hp.reduce())
    assert np.all(np.abs(bs - bp) <= 1e-5 * np.abs(bp) + 1e-12), (bs, bp)


def test_stream_one_step_against_oracle(native, orc):
    """One step from the same FP64 state, computed in FP32: per-link E change
    (the force) within FP32 rounding of the oracle's FP64 update."""
    dims = (4, 8, 32)
    g = fresh(oracle_ic(3, dims, 3, 0.3, 0.3, a=(1.0, 1.1, 0.9)))
    h = _handle(g, {"OPX_STREAM_FP32": "1"}, precision=N.OPX_F32, reunit_every=0)
    sim = orc.OracleSimulation(g)
    E0 = g.E.copy()
    sim.initialize()
    h.initialize()
    sim.step()
    h.step(1)
    e_gpu = h.download(N.FIELD_E)
    dref = (g.E - E0).reshape(-1, 9)
    dgpu = (e_gpu - E0).reshape(-1, 9)
    scale = np.abs(dref).max()
    assert np.abs(dgpu - dref).max() <= 3e-6 * scale + 2e-7
