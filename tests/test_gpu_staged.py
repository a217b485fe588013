"""The PCG's masked SpMV streams the operator through shared memory in tiles
of consecutive nodes.  These systems have ragged node degrees (hub nodes
with hundreds of neighbours next to nodes with five), so tiles start and end
at every alignment, some tiles exceed a stage and are read directly, and one
case passes CSR values that are not 16-byte aligned (no staging at all).
Solutions are checked against scipy's direct solve."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def stage_every_operator(monkeypatch):
    """These systems are L2-sized; stage them anyway (the library otherwise
    keeps operators below half of the L2 on the unstaged kernel)."""
    monkeypatch.setenv("GFEA_STAGE_MIN_BYTES", "0")


def hub_graph(Nn, hubs, hub_deg, seed):
    """Sorted neighbour lists (self included): a ring with +-2 neighbours and
    'hubs' consecutive nodes each joined to hub_deg random others."""
    rng = np.random.default_rng(seed)
    adj = [set([a, (a + 1) % Nn, (a - 1) % Nn, (a + 2) % Nn, (a - 2) % Nn]) for a in range(Nn)]
    h0 = Nn // 5
    for h in range(h0, h0 + hubs):
        for b in rng.choice(Nn, size=hub_deg, replace=False):
            adj[h].add(int(b))
            adj[int(b)].add(h)
    node_ptr = np.zeros(Nn + 1, np.int64)
    nbr = []
    for a in range(Nn):
        s = sorted(adj[a])
        nbr.extend(s)
        node_ptr[a + 1] = node_ptr[a] + len(s)
    return node_ptr.astype(np.int32), np.asarray(nbr, np.int32)


def spd_values(node_ptr, nbr, D, seed):
    """(L + shift I) kron M in the node-block CSR layout, with the scipy matrix."""
    import scipy.sparse as sp

    rng = np.random.default_rng(seed)
    Nn = len(node_ptr) - 1
    w = rng.uniform(0.5, 1.5, size=len(nbr))
    W = sp.csr_matrix((w, nbr, node_ptr), shape=(Nn, Nn))
    W = (W + W.T) * 0.5
    W.setdiag(0)
    W.eliminate_zeros()
    L = sp.diags(np.asarray(W.sum(axis=1)).ravel() + 0.05) - W
    B = rng.normal(size=(D, D))
    M = B @ B.T + D * np.eye(D)
    A = sp.kron(L.tocsr(), M).tocsr()
    # node-block CSR values: row (a, i), neighbour k, component j at
    # D^2 node_ptr[a] + i D nb(a) + D k + j
    Ld = L.tocsr()
    vals = np.zeros(D * D * len(nbr))
    for a in range(Nn):
        p0, p1 = node_ptr[a], node_ptr[a + 1]
        nb = p1 - p0
        lrow = Ld[a].toarray().ravel()
        for k in range(nb):
            blk = lrow[nbr[p0 + k]] * M
            for i in range(D):
                base = D * D * p0 + i * D * nb + D * k
                vals[base:base + D] = blk[i]
    return vals, A


def solve(node_ptr, nbr, vals, D, known, xk, b, precision, misalign=False):
    import torch

    from easyfea_gb300 import _lib

    dev = torch.device("cuda", 0)
    Nn = len(node_ptr) - 1
    np_d = torch.from_numpy(node_ptr).to(dev)
    nbr_d = torch.from_numpy(nbr).to(dev)
    if misalign:  # values at an 8-byte offset: not stageable
        buf64 = torch.zeros(len(vals) + 1, dtype=torch.float64, device=dev)
        v64 = buf64[1:]
        buf32 = torch.zeros(len(vals) + 2, dtype=torch.float32, device=dev)
        v32 = buf32[2:]
    else:
        v64 = torch.zeros(len(vals), dtype=torch.float64, device=dev)
        v32 = torch.zeros(len(vals), dtype=torch.float32, device=dev)
    v64.copy_(torch.from_numpy(vals))
    v32.copy_(v64.float())
    kn = torch.from_numpy(known.astype(np.uint8)).to(dev)
    x = torch.from_numpy(np.where(known, xk, 0.0)).to(dev)
    bd = torch.from_numpy(b).to(dev)
    L = _lib.load()
    sys = _lib.System(_lib.ABI_VERSION, D, Nn, len(nbr), _lib.ptr(np_d), _lib.ptr(nbr_d), _lib.ptr(v64),
                      _lib.ptr(v32), _lib.ptr(kn), 0, 0, None)
    prec = _lib.F64 if precision == "fp64" else _lib.F32
    opts = _lib.PcgOpts(_lib.ABI_VERSION, prec, 20000, 0, 1e-12, 0.0, 30, 0, 0, 0)
    ws = ctypes.c_size_t()
    _lib.check(L.gfea_pcg_workspace_size(ctypes.byref(sys), ctypes.byref(opts), ctypes.byref(ws)), "ws")
    work = torch.empty(int(ws.value), dtype=torch.uint8, device=dev)
    res = _lib.PcgResult()
    st = L.gfea_pcg_solve(ctypes.byref(sys), _lib.ptr(bd), _lib.ptr(x), ctypes.byref(opts), _lib.ptr(work),
                          work.numel(), ctypes.byref(res), _lib.stream())
    _lib.check(st, "pcg")
    return x.cpu().numpy(), res


@pytest.mark.parametrize("D", [1, 2, 3])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("misalign", [False, True])
def test_ragged_degrees_solution(D, precision, misalign):
    import scipy.sparse.linalg as spla

    Nn = 3000 if D < 3 else 1500
    node_ptr, nbr = hub_graph(Nn, hubs=12, hub_deg=300, seed=D)
    vals, A = spd_values(node_ptr, nbr, D, seed=10 + D)
    rng = np.random.default_rng(5)
    N = Nn * D
    known = np.zeros(N, bool)
    known[rng.choice(N, size=N // 50, replace=False)] = True
    xk = rng.normal(size=N)
    b = rng.normal(size=N)
    x, res = solve(node_ptr, nbr, vals, D, known, xk, b, precision, misalign)
    assert res.status == 0
    # reference: eliminate the known DOFs and solve the rest directly
    u = ~known
    Auu = A[u][:, u].tocsc()
    rhs = b[u] - A[u][:, known] @ xk[known]
    ref = spla.spsolve(Auu, rhs)
    assert np.array_equal(x[known], xk[known])
    resid = np.linalg.norm(rhs - Auu @ x[u]) / np.linalg.norm(rhs)
    assert resid <= 1e-10, resid
    err = np.abs(x[u] - ref).max() / np.abs(ref).max()
    assert err <= 1e-7, err
