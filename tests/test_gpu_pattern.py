"""Device sparsity pattern: bit-exact with the reference's scipy COO->CSR."""

import numpy as np
import pytest

from easyfea_gb300 import mesh as gmesh
from oracle import fem

pytestmark = pytest.mark.gpu

MESHES = {
    "quad4": lambda: gmesh.Mesh_Quad4_Rect(3.0, 2.0, 7, 5),
    "tri3": lambda: gmesh.Mesh_Tri3_Rect(3.0, 2.0, 6, 4),
    "quad9": lambda: gmesh.Mesh_Quad9_Rect(3.0, 2.0, 4, 3),
    "hexa8": lambda: gmesh.Mesh_Hexa8_Box(3.0, 2.0, 1.0, 5, 3, 2),
}


@pytest.mark.parametrize("name", list(MESHES))
def test_pattern_bit_exact(name):
    from easyfea_gb300.device import DeviceMesh

    m = MESHES[name]()
    dm = DeviceMesh(m)
    for dof_n in (1, m.dim):
        indptr, indices = dm.pattern(dof_n)
        inv, ind_ref, ptr_ref, nnz = fem.csr_map(np.asarray(m.connect), dof_n, m.Nn * dof_n)
        assert np.array_equal(indptr.cpu().numpy(), ptr_ref.astype(np.int64))
        assert np.array_equal(indices.cpu().numpy(), ind_ref)
        # slot map: CSR slot of element entry (p,i,q,j) from node_ptr + rank equals scipy's searchsorted
        node_ptr = dm.node_ptr.cpu().numpy().astype(np.int64)
        rank = dm.rank.cpu().numpy().reshape(m.Ne, m.groupElem.nPe, m.groupElem.nPe).astype(np.int64)
        con = np.asarray(m.connect)
        nPe = con.shape[1]
        nd = nPe * dof_n
        slots = np.empty((m.Ne, nd, nd), dtype=np.int64)
        for p in range(nPe):
            a = con[:, p]
            nb = node_ptr[a + 1] - node_ptr[a]
            for i in range(dof_n):
                base = dof_n * dof_n * node_ptr[a] + i * dof_n * nb
                for q in range(nPe):
                    for j in range(dof_n):
                        slots[:, p * dof_n + i, q * dof_n + j] = base + dof_n * rank[:, p, q] + j
        assert np.array_equal(slots.ravel(), inv.astype(np.int64))


def test_pattern_orphan_node():
    """A node used by no element has an empty row, as in scipy's pattern."""
    from easyfea_gb300.device import DeviceMesh
    from easyfea_gb300.mesh import ElemType, GroupElem, Mesh

    coord = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [5, 5, 0]], float)
    con = np.array([[0, 1, 2, 3]])
    m = Mesh({ElemType.QUAD4: GroupElem(ElemType.QUAD4, con, coord)})
    dm = DeviceMesh(m)
    indptr, indices = dm.pattern(2)
    inv, ind_ref, ptr_ref, nnz = fem.csr_map(con, 2, 10)
    assert np.array_equal(indptr.cpu().numpy(), ptr_ref.astype(np.int64))
    assert np.array_equal(indices.cpu().numpy(), ind_ref)
