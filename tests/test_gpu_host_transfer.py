"""Host transfers through page-locked buffers.

opx_upload / opx_download read and write a page-locked host buffer
(cudaMallocHost, here opx.PinnedArray) directly from the conversion kernels and
send pageable buffers through a device staging copy.  Both routes must give the
same device fields and the same host arrays, bit for bit, for every field,
layout, group and precision; a page-locked buffer of the wrong size is refused
like a pageable one.
"""
import numpy as np
import pytest

import openpixi_gb300 as opx
from openpixi_gb300 import _native as N

pytestmark = pytest.mark.gpu

FIELDS = [(N.FIELD_U, N.LAYOUT_REF), (N.FIELD_UNEXT, N.LAYOUT_REF), (N.FIELD_E, N.LAYOUT_REF),
          (N.FIELD_E, N.LAYOUT_GEN), (N.FIELD_J, N.LAYOUT_GEN), (N.FIELD_RHO, N.LAYOUT_GEN)]


def pinned_copy(a):
    p = opx.PinnedArray(a.shape)
    p.array[...] = a
    return p


@pytest.mark.parametrize("nc,prec,dims", [(3, N.OPX_F32, (6, 7, 9)), (3, N.OPX_F64, (5, 4, 6)),
                                          (2, N.OPX_F64, (9, 5, 7)), (2, N.OPX_F32, (4, 4, 33))])
def test_pinned_and_pageable_routes_agree(native, nc, prec, dims):
    ha = opx.Handle(nc, dims, precision=prec)
    hb = opx.Handle(nc, dims, precision=prec)
    ha.init_random(11, 0.3, 0.3)
    rng = np.random.default_rng(3)
    for field, layout in FIELDS:
        host = ha.download(field, layout=layout)        # pageable route
        if field in (N.FIELD_J, N.FIELD_RHO):
            host = rng.normal(0, 0.1, host.shape)
        pin = pinned_copy(host)
        ha.upload(field, host, layout=layout)           # pageable
        hb.upload(field, pin.array, layout=layout)      # page-locked, read by the kernel
        back_a = ha.download(field, layout=layout)
        out = opx.PinnedArray(host.shape)
        out.array[...] = np.nan
        hb.download(field, layout=layout, out=out.array)  # page-locked, written by the kernel
        assert np.array_equal(back_a, out.array), (field, layout)
        assert np.array_equal(hb.download(field, layout=layout), back_a), (field, layout)
        pin.free()
        out.free()
    ha.initialize()
    hb.initialize()
    ha.step(2)
    hb.step(2)
    oa, ob = ha.reduce(), hb.reduce()
    assert oa.e2_total == ob.e2_total and oa.b2_total == ob.b2_total and oa.gauss == ob.gauss


def test_pinned_wrong_size_refused(native):
    h = opx.Handle(2, (4, 4, 4))
    p = opx.PinnedArray((64 * 3 * 4 - 1,))
    with pytest.raises(opx.OpixiError) as e:
        h.upload(N.FIELD_U, p.array)
    assert e.value.code == N.OPX_ERR_INVALID
    p.free()
