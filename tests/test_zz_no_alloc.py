"""opx_reduce_noalloc: the reductions for callers that cannot allocate device
memory (their device memory belongs to another allocator, or they must not stall
on cudaMalloc).  The caller owns every device buffer -- here torch tensors stand
in for such a caller's memory -- and the entry point uses only the library's
fixed static scratch.  Its output must equal opx_reduce's (relative 1e-12) on
two calls in a row, since every call reuses the same scratch.

This file is collected last so that a stopped run has already run the others.
"""
import ctypes as C

import numpy as np
import pytest

import openpixi_gb300 as opx
from openpixi_gb300 import _native as N

pytestmark = pytest.mark.gpu

FIELDS = ("e2", "b2", "px", "py", "pz", "gauss", "rho2", "e2_total", "b2_total")


def as_vec(o):
    return np.array(list(o.e2) + list(o.b2) + [o.px, o.py, o.pz, o.gauss, o.rho2, o.e2_total, o.b2_total])


def planes(arr, ndir):
    """Host [V][ndir][k] -> device algebra layout [ndir][k][V] (contiguous)."""
    V = arr.shape[0]
    if ndir == 0:
        return np.ascontiguousarray(arr.T)
    return np.ascontiguousarray(arr.transpose(1, 2, 0)).reshape(-1, V)


def link_blocks(arr):
    """Host links [V][3][ng] -> device layout: SU(3) [3][ceil(V/32)][18][32],
    SU(2) [3][32 ceil(V/32)][4]."""
    V, _, ng = arr.shape
    nb = (V + 31) // 32
    pad = np.zeros((nb * 32, 3, ng))
    pad[:V] = arr
    if ng == 4:
        return np.ascontiguousarray(pad.transpose(1, 0, 2))
    return np.ascontiguousarray(pad.reshape(nb, 32, 3, ng).transpose(2, 0, 3, 1))


CASES = [(nc, prec, form) for nc in (2, 3) for prec in (N.OPX_F64, N.OPX_F32) for form in ("rho", "eval")]


@pytest.mark.parametrize("nc,prec,form", CASES)
def test_noalloc_matches_reduce(native, nc, prec, form):
    """form "rho": a charge density and every cell evaluated; form "eval": no
    charge (rho = NULL) and an evaluation mask, passed to both entry points."""
    torch = pytest.importorskip("torch")
    dims = (12, 10, 14)
    h = opx.Handle(nc, dims, dt=0.05, precision=prec, reunit_every=10 if prec == N.OPX_F32 else 0)
    h.init_random(31, 0.3, 0.3)
    h.gauss_project(1e-24)
    rng = np.random.default_rng(4)
    mask = None
    if form == "rho":
        rho = rng.normal(0, 0.05, (h.V, h.ngen))
        h.upload(N.FIELD_RHO, rho, layout=N.LAYOUT_GEN)
    else:
        mask = (rng.random(h.V) < 0.6).astype(np.uint8)
        h.set_evaluatable(mask)
    h.initialize()
    h.step(3)
    ref = as_vec(h.reduce())

    dt = torch.float32 if prec == N.OPX_F32 else torch.float64
    dev = torch.device("cuda", 0)
    U = torch.from_numpy(link_blocks(h.download(N.FIELD_U))).to(dev, dt)
    Un = torch.from_numpy(link_blocks(h.download(N.FIELD_UNEXT))).to(dev, dt)
    E = torch.from_numpy(planes(h.download(N.FIELD_E, layout=N.LAYOUT_GEN), 3)).to(dev, dt)
    R = None
    if form == "rho":
        R = torch.from_numpy(planes(h.download(N.FIELD_RHO, layout=N.LAYOUT_GEN), 0)).to(dev, dt)
    M = None if mask is None else torch.from_numpy(mask).to(dev)
    out = torch.full((13,), float("nan"), dtype=torch.float64, device=dev)
    dims_c = (C.c_int * 3)(*dims)
    a_c = (C.c_double * 3)(1.0, 1.0, 1.0)
    stream = torch.cuda.current_stream(dev).cuda_stream

    def call():
        return native.opx_reduce_noalloc(nc, prec, dims_c, a_c, 1.0, C.c_void_p(U.data_ptr()),
                                         C.c_void_p(Un.data_ptr()), C.c_void_p(E.data_ptr()),
                                         None if R is None else C.c_void_p(R.data_ptr()),
                                         None if M is None else C.c_void_p(M.data_ptr()),
                                         C.c_void_p(out.data_ptr()), C.c_void_p(stream))

    # a first call loads the kernels and looks up the scratch address; the two
    # calls checked after it must leave the device's free memory unchanged
    assert call() == N.OPX_OK
    torch.cuda.synchronize(dev)
    free_before = torch.cuda.mem_get_info(dev)[0]
    for _ in range(2):
        out.fill_(float("nan"))
        assert call() == N.OPX_OK
        torch.cuda.synchronize(dev)
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got))
        # FP32 storage: opx_reduce forms the per-site values with the paired
        # SU(3) FP32 kernel, in another operation order (FP32 rounding); the
        # Gauss column of a projected FP32 state without charge is rounding
        # noise (~1e-14), compared on the absolute scale of the energy
        if prec == N.OPX_F32:
            assert np.allclose(got, ref, rtol=1e-6, atol=1e-12 * abs(ref[-2] + ref[-1])), (got, ref)
        else:
            assert np.allclose(got, ref, rtol=1e-12, atol=1e-300), (got, ref)
    assert torch.cuda.mem_get_info(dev)[0] == free_before


def test_noalloc_rejects_oversize(native):
    """Sizes beyond the limit are refused before anything is launched; the
    buffers passed are real (small) device buffers all the same."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    buf = torch.zeros(64, dtype=torch.float64, device=dev)
    p = C.c_void_p(buf.data_ptr())
    dims_c = (C.c_int * 3)(1024, 1024, 1024)
    a_c = (C.c_double * 3)(1.0, 1.0, 1.0)
    rc = native.opx_reduce_noalloc(2, N.OPX_F64, dims_c, a_c, 1.0, p, p, p, None, None, p, None)
    assert rc == N.OPX_ERR_INVALID
    # a link buffer that is not 16-byte aligned is refused before any launch
    dims_s = (C.c_int * 3)(2, 2, 2)
    q = C.c_void_p(buf.data_ptr() + 8)
    rc = native.opx_reduce_noalloc(2, N.OPX_F64, dims_s, a_c, 1.0, q, p, p, None, None, p, None)
    assert rc == N.OPX_ERR_INVALID
