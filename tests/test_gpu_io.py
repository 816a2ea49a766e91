"""gs_set_field / gs_get_field with pinned host buffers (read and written by the permutation
kernels over the host link) against pageable ones (through the staging copy): the device
state and the fields read back are bit-identical, in both precisions, also for a field that
starts inside a larger pinned block."""
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import tables

pytestmark = pytest.mark.gpu
DZ = 2e-8   # one fixed step (m)
torch = pytest.importorskip("torch")


def setup(n_r=128, n_t=1024):
    d = tempfile.mkdtemp(prefix="gs_io_")
    p = configs.hot_solid(d, n_r=n_r, n_t=n_t, power_cr=20.0, tol=1e-2)
    return tables.build(tables.Config.from_file(p), noise_seed=3, noise_sigma=1e-4)


def within_low_parts(x, y):
    """Mixed handles carry BIGBUFFER2's window columns as double-float pairs; a state read back
    (high + low parts in FP64) and set again continues to within double-float rounding: the
    spectra may differ only below FP32 resolution, element by element."""
    return bool(np.all(np.abs(x - y) <= 2.0 ** -30 * np.abs(y)))


def pinned_like(a):
    t = torch.empty(a.shape, dtype=torch.complex128, pin_memory=True)
    t.numpy()[...] = a
    return t


@pytest.mark.parametrize("prec", [gs.PREC_MIXED, gs.PREC_FP64])
def test_pinned_and_pageable_agree(prec):
    T = setup()
    rng = np.random.default_rng(1)
    f = T["field"]
    s = rng.standard_normal(f.shape) + 1j * rng.standard_normal(f.shape)
    P = gs.Propagator(T, precision=prec)
    # pageable in, pageable out
    P.set_field(f, spec=s)
    P.nl_step(DZ)
    P.lstep(DZ)
    f_ref, s_ref = P.get_field(want_spec=True)
    # pinned in, pinned out
    fp, sp = pinned_like(f), pinned_like(s)
    P.set_field_ptr(fp.data_ptr(), sp.data_ptr())
    P.nl_step(DZ)
    P.lstep(DZ)
    fo = torch.zeros(f.shape, dtype=torch.complex128, pin_memory=True)
    so = torch.zeros(f.shape, dtype=torch.complex128, pin_memory=True)
    P.get_field_ptr(fo.data_ptr(), so.data_ptr())
    assert np.array_equal(fo.numpy(), f_ref)
    assert np.array_equal(so.numpy(), s_ref)
    # pinned in, pageable out and the reverse
    P.set_field_ptr(fp.data_ptr(), sp.data_ptr())
    a, b = P.get_field(want_spec=True)
    assert np.array_equal(a, f.astype(np.complex64).astype(np.complex128) if prec == gs.PREC_MIXED else f)
    P.set_field(f, spec=s)
    fo.zero_()
    P.get_field_ptr(fo.data_ptr(), None)
    assert np.array_equal(fo.numpy(), a)


def test_pinned_pointer_inside_a_larger_allocation():
    """A field that starts inside a larger pinned block (the second half of it): the range
    check measures from the pointer, the kernels read and write only the field's bytes."""
    T = setup(n_r=128, n_t=512)
    P = gs.Propagator(T, precision=gs.PREC_FP64)
    f = T["field"]
    P.set_field(f)
    ref = P.get_field(want_spec=False)
    n = f.shape[0]
    big = torch.zeros((2 * n, f.shape[1]), dtype=torch.complex128, pin_memory=True)
    big.numpy()[n:] = f
    P.set_field_ptr(big[n:].data_ptr(), None)
    assert np.array_equal(P.get_field(want_spec=False), ref)
    big.zero_()
    P.get_field_ptr(big[n:].data_ptr(), None)
    assert np.array_equal(big.numpy()[n:], ref)
    assert not big.numpy()[:n].any()   # nothing written before the pointer


def test_compact_spectrum_state_transitions():
    """BIGBUFFER2's window columns live in the mixed plan's compact copy between steps: reading
    the state after every step, replacing it mid-run, or reading it only at the end gives
    bit-identical fields and spectra."""
    T = setup(n_r=128, n_t=1024)
    f0 = T["field"]
    a = gs.Propagator(T, precision=gs.PREC_MIXED)
    b = gs.Propagator(T, precision=gs.PREC_MIXED)
    a.set_field(f0)
    b.set_field(f0)
    for _ in range(3):
        for P in (a, b):
            P.nl_step(DZ)
            P.lstep(DZ)
        fa, sa = a.get_field(want_spec=True)   # a is read back after every step
    fb, sb = b.get_field(want_spec=True)
    assert np.array_equal(fa, fb) and np.array_equal(sa, sb)
    # replace the state mid-run on one handle; a fresh handle started there agrees
    rng = np.random.default_rng(2)
    s_new = sb * (1 + 1e-3 * rng.standard_normal(sb.shape))
    b.set_field(fb, spec=s_new)
    c = gs.Propagator(T, precision=gs.PREC_MIXED)
    c.set_field(fb, spec=s_new)
    for P in (b, c):
        for _ in range(2):
            P.nl_step(DZ)
            P.lstep(DZ)
    fb2, sb2 = b.get_field(want_spec=True)
    fc2, sc2 = c.get_field(want_spec=True)
    assert np.array_equal(fb2, fc2) and np.array_equal(sb2, sc2)


def test_compact_field_state_transitions():
    """On grids whose NL step is the four-stage kernel of 16384-point rows, FIELD stays in the
    masked inverse's compact array between steps and the next NL step reads it there: reading
    the field after every step (which expands it), or only at the end, gives bit-identical
    fields and spectra; a handle restarted from the state read back continues with a
    bit-identical field and a spectrum equal to below FP32 resolution."""
    T = setup(n_r=640, n_t=16384)
    f0 = T["field"]
    a = gs.Propagator(T, precision=gs.PREC_MIXED)
    b = gs.Propagator(T, precision=gs.PREC_MIXED)
    a.set_field(f0)
    b.set_field(f0)
    for _ in range(3):
        for P in (a, b):
            P.nl_step(DZ)
            P.lstep(DZ)
        fa, sa = a.get_field(want_spec=True)
    fb, sb = b.get_field(want_spec=True)
    assert np.array_equal(fa, fb) and np.array_equal(sa, sb)
    # outside the spectral window the field read back is exactly zero, as the expansion writes it
    assert np.abs(fb).max() > 0
    c = gs.Propagator(T, precision=gs.PREC_MIXED)
    c.set_field(fb, spec=sb)
    for P in (b, c):
        P.nl_step(DZ)
        P.lstep(DZ)
    fb2, sb2 = b.get_field(want_spec=True)
    fc2, sc2 = c.get_field(want_spec=True)
    assert np.array_equal(fb2, fc2) and within_low_parts(sc2, sb2)


def test_compact_field_read_by_dumps_and_time_field():
    """The dump reductions and the time-domain field read FIELD itself: on a handle whose FIELD
    is compact they expand it first, and give what they give after an explicit read-back."""
    T = setup(n_r=640, n_t=16384)
    f0 = T["field"]
    a = gs.Propagator(T, precision=gs.PREC_MIXED)
    b = gs.Propagator(T, precision=gs.PREC_MIXED)
    a.set_field(f0)
    b.set_field(f0)
    for _ in range(2):
        for P in (a, b):
            P.nl_step(DZ)
            P.lstep(DZ)
    a.get_field(want_spec=False)   # a's FIELD expanded by the read-back
    da = a.dumps(T["qdht_x"], T["r_max"])
    db = b.dumps(T["qdht_x"], T["r_max"])   # b's expanded by the dump itself
    for k in da:
        assert np.array_equal(da[k], db[k]), k
    # both continue identically; the time-domain field agrees as well
    for P in (a, b):
        P.nl_step(DZ)
        P.lstep(DZ)
    assert np.array_equal(a.time_field(), b.time_field())
