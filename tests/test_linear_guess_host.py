"""LinearResponseGuess's regression on the host (torch on CPU, a stand-in engine): it recovers an exactly linear
density model from noiseless data, keeps the packed lower triangle symmetric on unpacking, and training in two
batches gives the same model as one."""
import numpy as np
import torch


class _Eng:
    def __init__(self, n_atoms, n_basis):
        self.n_atoms, self.n_basis, self.device = n_atoms, n_basis, torch.device("cpu")


def _data(rng, F, n, N, J, p0):
    x = rng.normal(scale=0.05, size=(F, n, 3)) + np.arange(n)[None, :, None]
    phi = rng.normal(scale=0.01, size=(F, n))
    f = np.concatenate([x.reshape(F, -1), phi], 1)
    pk = p0 + f @ J
    il = np.tril_indices(N)
    P = np.zeros((F, N, N))
    P[:, il[0], il[1]] = pk
    P[:, il[1], il[0]] = pk
    return torch.tensor(x), torch.tensor(phi), torch.tensor(P)


def test_linear_response_guess_recovers_a_linear_model():
    from pdynamo_mirror_gb300.guess import LinearResponseGuess
    rng = np.random.default_rng(3)
    n, N, F = 4, 6, 300
    J = rng.normal(size=(4 * n, N * (N + 1) // 2))
    p0 = rng.normal(size=N * (N + 1) // 2)
    x, phi, P = _data(rng, F, n, N, J, p0)
    g = LinearResponseGuess(_Eng(n, N), ridge=1e-9).fit(x, phi, P)
    xt, phit, Pt = _data(np.random.default_rng(4), 5, n, N, J, p0)
    Pp = g.predict(xt, phit)
    np.testing.assert_allclose(Pp.numpy(), Pt.numpy(), rtol=0, atol=2e-4)   # FP32 prediction GEMM
    np.testing.assert_array_equal(Pp.numpy(), np.transpose(Pp.numpy(), (0, 2, 1)))
    g2 = LinearResponseGuess(_Eng(n, N), ridge=1e-9)
    g2.fit(x[:100], phi[:100], P[:100]).fit(x[100:], phi[100:], P[100:])
    np.testing.assert_allclose(g2.predict(xt, phit).numpy(), Pp.numpy(), rtol=0, atol=1e-5)
    assert g.enabled and g.start_mode == 1
