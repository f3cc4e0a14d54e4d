"""Coulomb gauge and occupation numbers (SU(2)) on the GPU against the oracle,
through the C ABI: the reference's CoulombGaugeTest iteration counts, the
occupation numbers within 1e-9 of the largest and the energy density within
1e-10 (FFT rounding: cuFFT against numpy), the same number of Coulomb
iterations, and the handle's fields untouched."""
import ctypes as C

import numpy as np
import pytest

import openpixi_gb300 as opx
from openpixi_gb300 import _native as N

pytestmark = pytest.mark.gpu


def gauge_transform(g, psi):
    from oracle import lib, _p
    L = lib()
    L.orc_coulomb_apply.argtypes = [C.c_void_p] * 5
    L.orc_coulomb_apply(g.pp, _p(np.ascontiguousarray(psi)), _p(g.U), _p(g.Unext), _p(g.E))


def handle_of(g, precision=N.OPX_F64):
    h = opx.Handle(2, g.dims, a=g.a, dt=g.dt, g=g.g, precision=precision)
    h.upload(N.FIELD_U, g.U)
    h.upload(N.FIELD_UNEXT, g.Unext)
    h.upload(N.FIELD_E, g.E)
    return h


@pytest.mark.parametrize("f1,f2,expect", [((0, 0, 0), (0, 0, 0), 1), ((.1, 0, 0), (0, 0, 0), 2),
                                          ((.1, 0, 0), (0, .1, 0), 3)])
def test_coulomb_gauge_known_answers(native, orc, f1, f2, expect):
    g = orc.OracleGrid(2, (2, 2, 2), dt=0.1)
    psi = np.zeros((3, 8))
    psi[:, 0] = -np.array(f1)
    psi[:, 1] = -np.array(f2)
    gauge_transform(g, psi)
    h = handle_of(g)
    _, _, it, dv = h.occupation_numbers(with_n=False)
    assert dv < 1e-18
    if expect < 3:
        assert it == expect
    else:
        assert it > 2


def test_occupation_numbers_vs_oracle(native, orc):
    from oracle import occupation
    g = orc.OracleGrid(2, (8, 6, 10), dt=0.05, g=1.3)
    g.random_links(5, 0.15)
    g.random_e(5, 0.1)
    g.update_links()
    n_ref, e_ref, conv = occupation.occupation_numbers(g)
    h = handle_of(g)
    U0 = h.download(N.FIELD_U)
    n, e, it, dv = h.occupation_numbers()
    assert it == len(conv)
    assert np.abs(n - n_ref).max() <= 1e-9 * np.abs(n_ref).max()
    assert abs(e - e_ref) <= 1e-10 * abs(e_ref)
    assert np.array_equal(h.download(N.FIELD_U), U0)
    # an FP32 handle measures in FP64 on widened copies of its fields
    h32 = handle_of(g, precision=N.OPX_F32)
    n32, e32, _, _ = h32.occupation_numbers()
    assert abs(e32 - e_ref) <= 1e-5 * abs(e_ref)


def test_occupation_rejects_bad_options(native):
    h = opx.Handle(3, (4, 4, 4))
    with pytest.raises(opx.OpixiError):
        h.occupation_numbers(mirrored_direction=3)
    with pytest.raises(opx.OpixiError):
        h.occupation_numbers(windows=8)
    h2 = opx.Handle(2, (4, 4, 4), a=(1.0, 1.0, 0.5))
    with pytest.raises(opx.OpixiError):
        h2.occupation_numbers()  # one lattice spacing only, as in the reference


OPTION_CASES = {
    "mirrored_0": dict(mirrored_direction=0),
    "mirrored_2": dict(mirrored_direction=2),
    "gaussian": dict(window_flags=1, collision_time=0.0, collision_position=(4.0, 3.0, 5.0),
                     cone_velocity=(1.0, 0.0, 0.0)),
    "tukey": dict(window_flags=2, collision_time=0.0, collision_position=(4.0, 3.0, 5.0),
                  cone_velocity=(1.0, 0.0, 0.5), tukey_width=0.4),
    "cone": dict(window_flags=4, collision_time=0.0, collision_position=(4.0, 3.0, 5.0),
                 cone_velocity=(1.0, 1.0, 0.0)),
    "mirrored_all_windows": dict(mirrored_direction=0, window_flags=7, collision_time=0.0,
                                 collision_position=(4.0, 3.0, 5.0), cone_velocity=(1.0, 0.0, 1.0),
                                 tukey_width=0.5),
}


@pytest.mark.parametrize("case", sorted(OPTION_CASES))
def test_occupation_options_vs_oracle(native, orc, case):
    """The mirrored grid and the Gaussian, Tukey and cone windows
    (OccupationNumbersInTime.java:92-115, :164-201, :506-703) against the
    oracle: occupation numbers within 1e-9 of the largest, energy 1e-10."""
    from oracle import occupation
    opt = OPTION_CASES[case]
    g = orc.OracleGrid(2, (8, 6, 10), dt=0.5, g=1.1)
    g.random_links(7, 0.15)
    g.random_e(7, 0.1)
    g.update_links()
    h = handle_of(g)
    h.step(6)  # the windows use the grid's time, steps x dt = 3
    g.U[...] = h.download(N.FIELD_U)
    g.Unext[...] = h.download(N.FIELD_UNEXT)
    g.E[...] = h.download(N.FIELD_E)
    n_ref, e_ref, conv = occupation.occupation_numbers(g, time=6 * 0.5, **opt)
    kw = {("windows" if k == "window_flags" else k): v for k, v in opt.items()}
    n, e, it, dv = h.occupation_numbers(**kw)
    assert it == len(conv)
    assert np.abs(n - n_ref).max() <= 1e-9 * np.abs(n_ref).max()
    assert abs(e - e_ref) <= 1e-10 * abs(e_ref)


SU3_CASES = {
    "plain": dict(),
    "mirrored_1": dict(mirrored_direction=1),
    "gaussian_cone": dict(window_flags=5, collision_time=0.0, collision_position=(3.0, 2.0, 3.0),
                          cone_velocity=(1.0, 0.0, 1.0)),
}


@pytest.mark.parametrize("case", sorted(SU3_CASES))
def test_su3_occupation_vs_oracle(native, orc, case):
    """SU(3): the Coulomb gauge with the SU(3) logarithm and the occupation
    numbers (8 colours), with the mirrored grid and the windows, against the
    oracle: n within 1e-9 of the largest, energy 1e-10, the same iterations."""
    from oracle import occupation
    opt = SU3_CASES[case]
    g = orc.OracleGrid(3, (6, 5, 7), dt=0.5, g=1.2)
    g.random_links(9, 0.2)
    g.random_e(9, 0.15)
    g.update_links()
    h = opx.Handle(3, g.dims, a=g.a, dt=g.dt, g=g.g, precision=N.OPX_F64)
    h.upload(N.FIELD_U, g.U)
    h.upload(N.FIELD_UNEXT, g.Unext)
    h.upload(N.FIELD_E, g.E)
    h.step(4)
    g.U[...] = h.download(N.FIELD_U)
    g.Unext[...] = h.download(N.FIELD_UNEXT)
    g.E[...] = h.download(N.FIELD_E)
    n_ref, e_ref, conv = occupation.occupation_numbers(g, max_iter=60, goal=1e-16, time=4 * 0.5, **opt)
    kw = {("windows" if k == "window_flags" else k): v for k, v in opt.items()}
    n, e, it, dv = h.occupation_numbers(max_iter=60, accuracy_goal=1e-16, **kw)
    assert n.shape == (g.V, 8)
    assert it == len(conv)
    assert np.abs(n - n_ref).max() <= 1e-9 * np.abs(n_ref).max()
    assert abs(e - e_ref) <= 1e-10 * abs(e_ref)
