"""The hand-written adjoint through the C ABI (gs_gradient / gs_forward_fixed /
gs_adjoint_step).

* FP64 gradient vs the oracle's FP64 adjoint (which is itself checked against central
  differences of the oracle forward): <= 1e-9 relative L2.
* FP64 gradient vs central differences of the GPU FP64 forward along seeded directions.
* Mixed (split-FP16 QDHT, the linear step and BIGBUFFER2's cotangent in double-float as in the
  forward, FP32 NL) gradient: directional derivatives within 1e-4 relative of the FP64 central
  differences.
* checkpointing: every checkpoint stride gives the bit-identical gradient (both precisions);
  the default records every step during the forward when it fits in memory.
* A torch.autograd.Function over the C ABI (ctypes) whose backward is gs_gradient.
"""
import tempfile

import numpy as np
import pytest

import gsolver_gb300 as gs
from gsolver_gb300 import configs
from oracle import oracle, tables

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def hot(n_r=16, n_t=512, power_cr=20.0, seed=7, **over):
    d = tempfile.mkdtemp(prefix="gs_gadj_")
    p = configs.hot_solid(d, n_r=n_r, n_t=n_t, power_cr=power_cr, tol=1e-2)
    T = tables.build(tables.Config.from_file(p), noise_seed=seed, noise_sigma=1e-4)
    T.update(over)
    return T


def schedule(T, steps):
    dz0 = tables.init_zstep_kerr(T, T["field"]) if T["n2"] else 2e-7
    f = np.array([1.0, 0.9, 1.1, 0.95, 1.05])
    dz_rk = dz0 * f[np.arange(steps) % 5]
    dz_lin = dz0 * f[(np.arange(steps) + 1) % 5]
    return dz_rk, dz_lin


@pytest.mark.parametrize("power_cr,over", [
    (20.0, {}),
    (45.0, {}),                       # multiphoton loss on, density near rho_n
    (30.0, {"raman_fraction": 0.0}),
    (20.0, {"n2": 0.0}),              # plasma only (stiffer: lower power for the fixed dz)
])
def test_fp64_gradient_matches_oracle_adjoint(power_cr, over):
    T = hot(power_cr=power_cr, **over)
    dz_rk, dz_lin = schedule(T, 3)
    w = np.random.default_rng(5).random((T["n_r"], T["n_t"]))
    Jo, go = oracle.Oracle(T).gradient(T["field"], dz_rk, dz_lin, w)
    P = gs.Propagator(T, precision=gs.PREC_FP64)
    J, g = P.gradient(T["field"], dz_rk, dz_lin, w)
    assert abs(J - Jo) <= 1e-12 * Jo
    assert rel(g, go) < 1e-9


def test_adjoint_step_matches_oracle():
    T = hot(power_cr=30.0)
    O = oracle.Oracle(T)
    dz_rk, dz_lin = schedule(T, 1)
    rng = np.random.default_rng(8)
    fb = rng.standard_normal(T["field"].shape) + 1j * rng.standard_normal(T["field"].shape)
    sb = rng.standard_normal(T["field"].shape) + 1j * rng.standard_normal(T["field"].shape)
    # the oracle's one-step adjoint
    s_ref, b1 = O.lstep_vjp(O.qdht_t(fb), sb, dz_lin[0])
    a_ref = O.nl_step_vjp(T["field"], dz_rk[0], O.qdht_t(b1))
    P = gs.Propagator(T, precision=gs.PREC_FP64)
    P.set_field(T["field"])
    a, s = P.adjoint_step(dz_rk[0], dz_lin[0], fb, sb)
    assert rel(a, a_ref) < 1e-9
    assert rel(s, s_ref) < 1e-12


@pytest.mark.parametrize("prec,n_r", [(gs.PREC_FP64, 32), (gs.PREC_MIXED, 128)])
def test_checkpoint_strides_give_identical_gradients(prec, n_r):
    """Re-run segments repeat the forward exactly: the mixed path's checkpoints hold BIGBUFFER2's
    double-float window columns too (128 rows: the tensor-core QDHT with its compact state)."""
    T = hot(n_r=n_r, n_t=1024, power_cr=30.0)
    dz_rk, dz_lin = schedule(T, 7)
    w = np.random.default_rng(1).random((T["n_r"], T["n_t"]))
    P = gs.Propagator(T, precision=prec)
    ref = None
    for k in (0, 1, 2, 3, 7):   # 0: every step recorded in the forward (a few MB here)
        J, g = P.gradient(T["field"], dz_rk, dz_lin, w, checkpoint_stride=k)
        assert P.adjoint_stride() == (k if k else 7)
        if ref is None:
            ref = (J, g)
        assert J == ref[0] and np.array_equal(g, ref[1])
    # the forward alone gives the same objective and leaves the final field
    Jf, f = P.forward_fixed(T["field"], dz_rk, dz_lin, w)
    assert Jf == ref[0]
    assert np.array_equal(f, P.get_field(want_spec=False))


def _band_weights(T, lo_nm, hi_nm):
    """average_spectrum radial weights (dump_types.cpp:427-457) on a spectral band."""
    c = 299792458.0
    om = np.asarray(T["omega"])
    band = (om >= 2 * np.pi * c / (hi_nm * 1e-9)) & (om <= 2 * np.pi * c / (lo_nm * 1e-9))
    x = np.asarray(T["qdht_x"])
    wr = np.empty_like(x)
    wr[0] = x[0] * (x[1] - x[0])
    wr[1:] = x[1:] * (x[1:] - x[:-1])
    return np.outer(wr * T["r_max"] ** 2 / 2, band.astype(float))


def test_gradients_vs_central_differences_fp64_and_mixed():
    T = hot(n_r=128, n_t=1024, power_cr=30.0, seed=3)   # the tensor-core QDHT takes n_r % 128 == 0
    dz_rk, dz_lin = schedule(T, 10)
    w = _band_weights(T, 600, 760)
    A0 = T["field"]
    P64 = gs.Propagator(T, precision=gs.PREC_FP64)
    J, g64 = P64.gradient(A0, dz_rk, dz_lin, w)
    Pm = gs.Propagator(T, precision=gs.PREC_MIXED)
    Jm, gm = Pm.gradient(A0, dz_rk, dz_lin, w)
    assert abs(Jm - J) <= 1e-4 * J
    assert rel(gm, g64) < 5e-5   # 2.0e-5 measured (10 steps of a strongly ionizing pulse)
    rng = np.random.default_rng(4)
    scale = np.linalg.norm(A0)
    # fourth-order central differences at h = 1e-5 (the h^2 term of the two-point rule is
    # ~1e-5 here).  The map is only piecewise smooth (the rate table is log-linear between
    # nodes), so differences taken across nodes average the slopes on both sides: on this
    # hot grid they settle ~1e-5 from the exact derivative (the oracle's adjoint shows the
    # same offset), which bounds what they can pin.
    h = 1e-5

    def Jf(A):
        return P64.forward_fixed(A, dz_rk, dz_lin, w)[0]

    for _ in range(3):
        v = rng.standard_normal(A0.shape) + 1j * rng.standard_normal(A0.shape)
        v *= scale / np.linalg.norm(v)
        fd = (-Jf(A0 + 2 * h * v) + 8 * Jf(A0 + h * v) - 8 * Jf(A0 - h * v) + Jf(A0 - 2 * h * v)) / (12 * h)
        d64 = float(np.sum((np.conj(g64) * v).real))
        dm = float(np.sum((np.conj(gm) * v).real))
        assert abs(d64 - fd) <= 3e-5 * abs(fd), (d64, fd)
        assert abs(dm - fd) <= 1e-4 * abs(fd), (dm, fd)


def test_torch_autograd_function_over_the_c_abi():
    torch = pytest.importorskip("torch")
    T = hot(n_r=16, n_t=512, power_cr=30.0)
    dz_rk, dz_lin = schedule(T, 4)
    w = np.random.default_rng(9).random((T["n_r"], T["n_t"]))
    P = gs.Propagator(T, precision=gs.PREC_FP64)

    class BandEnergy(torch.autograd.Function):
        """J(FIELD_0) through gs_forward_fixed; backward through gs_gradient (ctypes)."""

        @staticmethod
        def forward(ctx, field):
            a = field.detach().cpu().numpy()
            ctx.save_for_backward(field)
            J, _ = P.forward_fixed(a, dz_rk, dz_lin, w)
            return field.new_tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gJ):
            (field,) = ctx.saved_tensors
            _, g = P.gradient(field.detach().cpu().numpy(), dz_rk, dz_lin, w)
            return gJ * torch.from_numpy(g).to(field.device)

    x = torch.tensor(T["field"], dtype=torch.complex128, requires_grad=True)
    J = BandEnergy.apply(x)
    (gx,) = torch.autograd.grad(J, x)
    _, g = P.gradient(T["field"], dz_rk, dz_lin, w)
    assert np.array_equal(gx.numpy(), g)
    # torch's convention for a real loss of a complex input is dJ/dRe + i dJ/dIm, as here:
    # a first-order step along -g lowers J
    with torch.no_grad():
        J2 = BandEnergy.apply(x - 1e-7 * J / torch.linalg.vector_norm(gx) ** 2 * gx)
    assert float(J2) < float(J.detach())


def test_package_autograd_objective_matches_the_adjoint():
    torch = pytest.importorskip("torch")
    from gsolver_gb300 import autograd as ga
    T = hot(n_r=16, n_t=512, power_cr=30.0)
    dz_rk, dz_lin = schedule(T, 4)
    w = np.random.default_rng(9).random((T["n_r"], T["n_t"]))
    P = gs.Propagator(T, precision=gs.PREC_FP64)
    J_of = ga.objective(P, dz_rk, dz_lin, w)
    x = torch.tensor(T["field"], dtype=torch.complex128, requires_grad=True)
    J = J_of(x)
    (gx,) = torch.autograd.grad(J, x)
    J_ref, g = P.gradient(T["field"], dz_rk, dz_lin, w)
    assert float(J) == pytest.approx(J_ref, rel=1e-12) and np.array_equal(gx.numpy(), g)
    P.close()
