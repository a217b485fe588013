"""Phase-field split kernel (gfea_pf_split) against the reference's Calc_C."""

import ctypes

import numpy as np
import pytest

from oracle import fem

pytestmark = pytest.mark.gpu


def gpu_split(eps, split, dim, planeStress):
    import torch

    from easyfea_gb300 import _lib

    L = _lib.load()
    lmbda, mu = fem.lame(210000.0, 0.3, dim, planeStress)
    C = fem.isotropic_C(210000.0, 0.3, dim, planeStress)
    p = _lib.PfParams()
    p.version = _lib.ABI_VERSION
    p.split = _lib.SPLIT_CODE[split]
    p.regularization = 1
    p.dim = dim
    p.lambda_ = float(lmbda)
    p.mu = float(mu)
    p.Gc, p.l0, p.thickness, p.k_res = 2.7, 0.01, 1.0, 1e-12
    p.plane_stress = int(planeStress)
    for i, v in enumerate(C.ravel()):
        p.C[i] = v
    n = 3 if dim == 2 else 6
    e = torch.as_tensor(np.ascontiguousarray(eps.reshape(-1, n)), device="cuda")
    npt = e.shape[0]
    cP = torch.empty(npt, n, n, dtype=torch.float64, device="cuda")
    cM = torch.empty_like(cP)
    psiP = torch.empty(npt, dtype=torch.float64, device="cuda")
    psiM = torch.empty_like(psiP)
    _lib.check(L.gfea_pf_split(_lib.ptr(e), npt, ctypes.byref(p), _lib.ptr(cP), _lib.ptr(cM), _lib.ptr(psiP),
                               _lib.ptr(psiM), _lib.stream()), "split")
    return cP.cpu().numpy(), cM.cpu().numpy(), psiP.cpu().numpy(), psiM.cpu().numpy(), C


@pytest.mark.parametrize("dim,ps", [(2, 1), (2, 0), (3, 0)])
@pytest.mark.parametrize("split", ["Bourdin", "Amor", "Miehe", "Zhang", "Stress", "He"])
def test_split_matches_reference(golden, dim, ps, split):
    g = golden("split")
    eps = g[f"d{dim}_eps"]
    key = f"d{dim}_ps{ps}_{split}"
    cP, cM, psiP, psiM, C = gpu_split(eps, split, dim, bool(ps))
    n = cP.shape[-1]
    refP = np.broadcast_to(g[key + "_cP"].reshape(-1, n, n), cP.shape)
    refM = np.broadcast_to(g[key + "_cM"].reshape(-1, n, n), cM.shape)
    scale = np.abs(C).max()
    lmbda, mu = fem.lame(210000.0, 0.3, dim, bool(ps))
    kw = dict(E=210000.0, v=0.3, planeStress=bool(ps))
    fP, _ = fem.split_C(eps, split, lmbda, mu, dim, C, robust=False, **kw)
    rP, rM = fem.split_C(eps, split, lmbda, mu, dim, C, robust=True, **kw)
    # degenerate rows (exactly repeated or zero eigenvalues): the reference
    # returns NaN, or its result depends on the last bit of a rounding residue
    bad = np.isnan(refP.reshape(len(cP), -1)).any(1) | \
        (np.abs(np.nan_to_num(fP, nan=1e300) - rP).reshape(len(cP), -1).max(1) > 1e-9 * scale)
    # only the special strains appended to the seeded ones can be degenerate
    n_special = 9 if dim == 3 else 6
    assert not bad[:-n_special].any()
    ok = ~bad
    assert np.max(np.abs(cP[ok] - refP[ok])) <= 1e-12 * scale
    assert np.max(np.abs(cM[ok] - refM[ok])) <= 1e-12 * scale
    gp = g[key + "_psiP"].reshape(-1)
    gm = g[key + "_psiM"].reshape(-1)
    s = np.abs(gp[ok]).max() + np.abs(gm[ok]).max()
    assert np.max(np.abs(psiP[ok] - gp[ok])) <= 1e-12 * s
    assert np.max(np.abs(psiM[ok] - gm[ok])) <= 1e-12 * s
    if bad.any():
        # degenerate rows follow the robust oracle and keep the split identities
        assert not np.isnan(cP[bad]).any()
        np.testing.assert_allclose(cP[bad], rP.reshape(cP.shape)[bad], atol=1e-9 * scale)
        np.testing.assert_allclose(cM[bad], rM.reshape(cM.shape)[bad], atol=1e-9 * scale)
        np.testing.assert_allclose(cP[bad] + cM[bad], np.broadcast_to(C, cP[bad].shape), atol=1e-9 * scale)


def test_split_identities_random_3d():
    """cP + cM = C and psi+ + psi- = psi on random 3D strains (property of the split)."""
    rng = np.random.default_rng(11)
    eps = rng.standard_normal((2000, 6)) * 1e-3
    cP, cM, psiP, psiM, C = gpu_split(eps, "Miehe", 3, False)
    np.testing.assert_allclose(cP + cM, np.broadcast_to(C, cP.shape), atol=1e-9 * np.abs(C).max())
    psi = 0.5 * np.einsum("pi,ij,pj->p", eps, C, eps)
    np.testing.assert_allclose(psiP + psiM, psi, rtol=1e-10, atol=1e-16)
    assert np.all(psiP >= -1e-12 * np.abs(psi).max())
