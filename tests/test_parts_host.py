"""The row-owned assembly's plan (gfea_part_plan_host, a host function of the
library, no GPU call): parts, node offsets and visit lists."""

import numpy as np
import pytest
import scipy.sparse as sp


def node_ptr_of(connect, Nn):
    """Node graph row pointers: neighbours (nodes sharing an element, the node
    itself included) of every node."""
    Ne, nPe = connect.shape
    inc = sp.csr_matrix((np.ones(connect.size), (connect.ravel(), np.repeat(np.arange(Ne), nPe))), shape=(Nn, Ne))
    A = (inc @ inc.T).tocsr()
    return np.concatenate([[0], np.cumsum(np.diff(A.indptr))]).astype(np.int32)


def meshes():
    from easyfea_gb300 import mesh as gmesh

    return {"quad4": gmesh.Mesh_Quad4_Rect(12.0, 3.0, 30, 8), "tri3": gmesh.Mesh_Tri3_Rect(1.0, 1.0, 12, 12),
            "quad9": gmesh.Mesh_Quad9_Rect(6.0, 2.0, 8, 4), "hexa8": gmesh.Mesh_Hexa8_Box(4.0, 1.0, 1.0, 12, 4, 4),
            "tetra4": gmesh.Mesh_Tetra4_Box(3.0, 1.0, 1.0, 6, 3, 3)}


@pytest.mark.parametrize("name", ["quad4", "tri3", "quad9", "hexa8", "tetra4"])
@pytest.mark.parametrize("max_values", [600, 5000])
def test_part_plan_invariants(name, max_values):
    from easyfea_gb300.device import part_plan_host

    m = meshes()[name]
    connect = m.groupElem.connect.astype(np.int32)
    Nn, (Ne, nPe) = m.Nn, connect.shape
    dof = m.dim
    node_ptr = node_ptr_of(connect, Nn)
    h = part_plan_host(m.coord, connect, node_ptr, dof, max_values)
    P = len(h["part_nvals"])
    vals = dof * dof * np.diff(node_ptr)
    # every node in exactly one part; offsets are the running sums of its rows
    assert sorted(h["part_nodes"].tolist()) == list(range(Nn))
    assert h["part_node_ptr"][0] == 0 and h["part_node_ptr"][-1] == Nn and np.all(np.diff(h["part_node_ptr"]) > 0)
    part_of = np.empty(Nn, int)
    for k in range(P):
        nodes = h["part_nodes"][h["part_node_ptr"][k]:h["part_node_ptr"][k + 1]]
        part_of[nodes] = k
        off = np.concatenate([[0], np.cumsum(vals[nodes])[:-1]])
        assert np.array_equal(h["node_off"][nodes], off)
        assert h["part_nvals"][k] == vals[nodes].sum() <= max_values
    # one visit per (element, part of one of its nodes); the masks cover every local node once
    cover = np.zeros((Ne, nPe), int)
    for k in range(P):
        el = h["visit_elem"][h["visit_ptr"][k]:h["visit_ptr"][k + 1]]
        mk = h["visit_mask"][h["visit_ptr"][k]:h["visit_ptr"][k + 1]]
        # by descending number of owned rows, then ascending element
        key = np.stack([-np.array([bin(int(x)).count("1") for x in mk]), el], 1)
        assert all(tuple(key[i]) < tuple(key[i + 1]) for i in range(len(key) - 1))
        for e, msk in zip(el, mk):
            bits = [(int(msk) >> p) & 1 for p in range(nPe)]
            assert all(part_of[connect[e, p]] == k for p in range(nPe) if bits[p])
            assert all(part_of[connect[e, p]] != k for p in range(nPe) if not bits[p])
            cover[e] += bits
    assert np.all(cover == 1)


def test_parts_are_compact():
    """Morton-ordered parts of 19,456 values (the FP32 part size): a HEXA8
    element is visited by fewer than two parts on average, a QUAD4 element by
    about one."""
    from easyfea_gb300 import mesh as gmesh
    from easyfea_gb300.device import part_plan_host

    for m, bound in ((gmesh.Mesh_Hexa8_Box(4.0, 1.0, 1.0, 40, 10, 10), 1.9),
                     (gmesh.Mesh_Quad4_Rect(12.0, 3.0, 120, 30), 1.1)):
        connect = m.groupElem.connect.astype(np.int32)
        h = part_plan_host(m.coord, connect, node_ptr_of(connect, m.Nn), m.dim, 19456)
        assert len(h["visit_elem"]) / len(connect) < bound


def test_part_plan_rejects_rows_larger_than_a_part():
    from easyfea_gb300.device import part_plan_host

    m = meshes()["hexa8"]
    connect = m.groupElem.connect.astype(np.int32)
    node_ptr = node_ptr_of(connect, m.Nn)
    with pytest.raises(RuntimeError):
        part_plan_host(m.coord, connect, node_ptr, 3, 200)  # an interior HEXA8 node has 243 values
