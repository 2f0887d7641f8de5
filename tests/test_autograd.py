"""The REML log-likelihood gradient through torch.autograd (test harness in reml_autograd.py):
backward = the GPU adjoint through the C ABI, checked against central differences of the exact
FP64 log-likelihood; the same check with the oracle's Hutchinson estimate pins the tolerance on
the CPU with the very probes the GPU draws."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from reml_autograd import REMLLogLikelihood, check_against_finite_differences, oracle_grad_fn, problem  # noqa: E402

SEEDS = list(range(16))
N_V = 256
SG2, SE2 = 0.55, 0.8


def _theta(wwin):
    return torch.tensor([SG2, SE2, *wwin.astype(np.float64)], dtype=torch.float64)


def test_oracle_estimate_through_autograd_vs_finite_differences():
    model, wwin = problem()
    model.update(seeds=SEEDS, grad_fn=oracle_grad_fn(model, N_V))
    check_against_finite_differences(model, _theta(wwin))


def _gpu_model():
    from slemm_gb300 import api, synth
    model, wwin = problem()
    g = api.Genotypes(synth.encode_bed(model["counts"]), model["counts"].shape[1])

    def fn(t, seed):
        r = g.REML_grad(model["rvec"], model["X"], model["y"], model["persnp"], model["window"],
                        t[2:].astype(np.float32), t[0], t[1], n_V=N_V, seed=seed, tol=1e-6)
        return np.concatenate([[r["d_sigma_g2"], r["d_sigma_e2"]], r["d_w"]])
    model.update(seeds=SEEDS, grad_fn=fn)
    return model, wwin, g


@pytest.mark.gpu
def test_gpu_adjoint_through_autograd(gpu):
    """backward() hands torch exactly the C-ABI gradient (mean over the probe seeds), and that
    gradient agrees with the oracle's estimate on the same probes."""
    model, wwin, g = _gpu_model()
    try:
        th = _theta(wwin).requires_grad_(True)
        REMLLogLikelihood.apply(th, model).backward()
        t = _theta(wwin).numpy()
        direct = np.mean([model["grad_fn"](t, s) for s in SEEDS], axis=0)
        assert np.allclose(th.grad.numpy(), direct, rtol=1e-12, atol=0)
        ref = np.mean([oracle_grad_fn(model, N_V)(t, s) for s in SEEDS], axis=0)
        assert abs(direct[0] - ref[0]) <= 2e-3 * abs(ref[0])
        assert abs(direct[1] - ref[1]) <= 2e-3 * abs(ref[1])
        assert np.max(np.abs(direct[2:] - ref[2:])) <= 2e-3 * np.max(np.abs(ref[2:]))
    finally:
        g.close()


@pytest.mark.gpu
def test_gpu_adjoint_through_autograd_vs_finite_differences(gpu):
    model, wwin, g = _gpu_model()
    try:
        check_against_finite_differences(model, _theta(wwin))
    finally:
        g.close()
