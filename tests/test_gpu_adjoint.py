"""The likelihood adjoint kernel (no reference counterpart): against the FP64
oracle (oracle/strip_oracle.c orc_nll_grad), central finite differences of the
GPU loss, the torch.autograd binding, and detector-resolution recalibration."""
import numpy as np
import pytest

import oracle as O
from jpet_strip import capi, phantom

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _setup(golden, n=4000, iters=2):
    manifest, load = golden
    g = manifest["c1"]["geometry"]
    args = (g["R"], g["L"], g["n_y"], g["n_z"], g["p"], g["sz"], g["sdl"])
    ev = load("c1_events.npy")[:n]
    rho, _ = O.mlem_f(O.Geometry(*args), ev, iters, threads=4)
    return capi.Geometry(*args), O.Geometry(*args), ev, rho


def test_loss_and_gradients_match_fp64_oracle(golden):
    cg, og, ev, rho = _setup(golden)
    with capi.StripReconstruction(cg) as rec:
        rec.set_events(ev)
        rho_d = torch.from_numpy(rho).cuda()
        grad = torch.empty_like(rho_d)
        torch.cuda.synchronize()
        for sig in [(og.sigma_z, og.sigma_dl), (11.0, 40.0)]:
            loss, gs, skipped = rec.nll_grad(sig[0], sig[1], rho_d.data_ptr(), None,
                                             grad.data_ptr())
            og2 = O.Geometry(og.radius, og.length, og.n_y, og.n_z, og.pixel, *sig)
            want_loss, want_grad, want_gs, want_sk = O.nll_grad(
                og2, ev, rho, support_sigma=(og.sigma_z, og.sigma_dl))
            assert skipped == want_sk
            assert abs(loss - want_loss) <= 1e-6 * abs(want_loss), (loss, want_loss)
            np.testing.assert_allclose(gs, want_gs, rtol=2e-4)
            g = grad.cpu().numpy().astype(np.float64)
            assert np.linalg.norm(g - want_grad) / np.linalg.norm(want_grad) < 1e-5


def test_sigma_gradient_matches_central_differences(golden):
    cg, og, ev, rho = _setup(golden)
    h = 1e-3
    with capi.StripReconstruction(cg) as rec:
        rec.set_events(ev)
        rho_d = torch.from_numpy(rho).cuda()
        torch.cuda.synchronize()
        s0 = np.array([og.sigma_z, og.sigma_dl])
        _, gs, _ = rec.nll_grad(*s0, rho_d.data_ptr())
        for i in range(2):
            sp, sm = s0.copy(), s0.copy()
            sp[i] += h
            sm[i] -= h
            fd = (rec.nll_grad(*sp, rho_d.data_ptr())[0] - rec.nll_grad(*sm, rho_d.data_ptr())[0]) / (2 * h)
            assert abs(fd - gs[i]) <= 2e-3 * max(abs(fd), 1.0), (i, fd, gs[i])


def test_autograd_function(golden):
    from jpet_strip.autograd import StripNLL

    cg, og, ev, rho = _setup(golden, n=2000)
    with capi.StripReconstruction(cg) as rec:
        rec.set_events(ev)
        rho_t = torch.from_numpy(rho).cuda().requires_grad_(True)
        sig = torch.tensor([og.sigma_z, og.sigma_dl], dtype=torch.float64, requires_grad=True)
        loss = StripNLL.apply(rho_t, sig, rec)
        loss.backward()
        want_loss, want_grad, want_gs, _ = O.nll_grad(og, ev, rho)
        assert abs(loss.item() - want_loss) <= 1e-6 * abs(want_loss)
        np.testing.assert_allclose(sig.grad.numpy(), want_gs, rtol=2e-4)
        g = rho_t.grad.cpu().numpy().astype(np.float64)
        assert np.linalg.norm(g - want_grad) / np.linalg.norm(want_grad) < 1e-5


def test_sigma_calibration_recovers_true_widths():
    """5e6 events of a centred point source simulated with sigma (10, 42) on the
    2 mm grid; gradient descent on sigma from (14, 55) with the source image known."""
    from jpet_strip.autograd import calibrate_sigma

    ev = phantom.generate_events(phantom.point_source(), 5_000_000, 450.0, 1000.0, 10.0, 42.0,
                                 seed=41)
    geom = capi.Geometry(450.0, 1000.0, 450, 500, 2.0, 14.0, 55.0)
    img = phantom.point_image(450, 500, 2.0, [(-1.0, -1.0)])
    sigma, hist = calibrate_sigma(geom, ev, img, (14.0, 55.0))
    assert abs(sigma[0] - 10.0) < 0.5 and abs(sigma[1] - 42.0) < 0.5, hist
    # the loss decreases along the descent
    losses = [h["loss"] for h in hist]
    assert all(b <= a + 1e-6 * abs(a) for a, b in zip(losses, losses[1:])), losses


def test_blind_recalibration_moves_towards_true_widths():
    """The blind form (MLEM image at the current widths, fit on held-out events)
    lowers both widths from (14, 55); it is not required to stop at the truth."""
    from jpet_strip.autograd import recalibrate_sigma

    ev = phantom.generate_events(phantom.three_ellipse_phantom(), 200000, 450.0, 1000.0, 10.0,
                                 42.0, seed=33)
    geom = capi.Geometry(450.0, 1000.0, 180, 200, 5.0, 14.0, 55.0)
    sigma, hist = recalibrate_sigma(geom, ev, (14.0, 55.0), outer=2)
    assert sigma[0] < 14.0 and sigma[1] < 55.0, hist


def _config3(n=6000):
    """The differentiable configuration's grid and widths: 500 x 450 at 2 mm,
    events simulated with sigma (10, 42), supports and image at (14, 55)."""
    args = (450.0, 1000.0, 450, 500, 2.0, 14.0, 55.0)
    ev = phantom.generate_events(phantom.random_ellipse_phantom(seed=3), n, 450.0, 1000.0,
                                 10.0, 42.0, seed=3)
    og = O.Geometry(*args)
    rho, _ = O.mlem_f(og, ev, 2, threads=8)
    return capi.Geometry(*args), og, ev, rho


def test_config3_grid_gradients_match_fp64_oracle_and_differences():
    cg, og, ev, rho = _config3()
    h = 1e-3
    with capi.StripReconstruction(cg) as rec:
        rec.set_events(ev)
        rho_d = torch.from_numpy(rho).cuda()
        grad = torch.empty_like(rho_d)
        torch.cuda.synchronize()
        loss, gs, skipped = rec.nll_grad(14.0, 55.0, rho_d.data_ptr(), None, grad.data_ptr())
        want_loss, want_grad, want_gs, want_sk = O.nll_grad(og, ev, rho)
        assert skipped == want_sk
        assert abs(loss - want_loss) <= 1e-6 * abs(want_loss), (loss, want_loss)
        np.testing.assert_allclose(gs, want_gs, rtol=2e-4)
        g = grad.cpu().numpy().astype(np.float64)
        # dL/drho = s - sum_e K_e / den_e nearly cancels once rho is close to the
        # MLEM fixed point, which amplifies the FP32 image's relative error
        # (measured 1.2e-5 here, 1700 support pixels per event)
        assert np.linalg.norm(g - want_grad) / np.linalg.norm(want_grad) < 5e-5
        s0 = np.array([14.0, 55.0])
        for i in range(2):
            sp, sm = s0.copy(), s0.copy()
            sp[i] += h
            sm[i] -= h
            fd = (rec.nll_grad(*sp, rho_d.data_ptr())[0] -
                  rec.nll_grad(*sm, rho_d.data_ptr())[0]) / (2 * h)
            assert abs(fd - gs[i]) <= 2e-3 * max(abs(fd), 1.0), (i, fd, gs[i])
