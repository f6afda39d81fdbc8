"""Host-side logic of the batched solver and the adjoint (no GPU): the union
layout of a batch and the parameter mapping of the misfit."""
import numpy as np

import oracle
from poromec_gb300 import meshgen


def test_batch_union_layout_contiguous_equations():
    """The union of a batch numbers each instance's equations as one
    contiguous range (what the batched solver's segmented layout relies on)."""
    ins = meshgen.batch_instances(ninst=5, nmin=2, nmax=5, seed=11)
    pb = meshgen.union_problem(ins)
    ptr = pb["inst_node_ptr"]
    assert ptr[0] == 0 and ptr[-1] == pb["nnode"] and len(ptr) == 6
    # each element lies inside one instance and carries its instance's material
    for k in range(5):
        sel = pb["ix"][:, 20] == k + 1
        nodes = pb["ix"][sel, :20] - 1
        assert nodes.min() >= ptr[k] and nodes.max() < ptr[k + 1]
    o = oracle.Oracle(int(pb["nnode"]), int(pb["nnodev"]), int(pb["numel"]), 20, 8, pb["ix"],
                      pb["id"], pb["fnno"], pb["x"], pb["ie"], pb["e"])
    idr = o.get_id()
    hi = 0
    for k in range(5):
        e = idr[ptr[k]:ptr[k + 1]]
        e = e[e > 0]
        assert e.min() == hi + 1 and e.max() - e.min() + 1 == len(e)
        hi = e.max()
    assert hi == o.neq


def test_batch_instances_seeded():
    a = meshgen.batch_instances(ninst=4, nmin=8, nmax=32, seed=4242)
    b = meshgen.batch_instances(ninst=4, nmin=8, nmax=32, seed=4242)
    assert [p["n"] for p in a] == [p["n"] for p in b]
    assert all(8 <= p["n"] <= 32 for p in a)
    assert np.array_equal(a[0]["e"], b[0]["e"])


def test_adjoint_parameter_mapping():
    """theta = (log E, log c_k, log M) per element maps back onto material
    columns 1, 3 and 4 exactly (the sweep's derivatives are with respect to
    these logs)."""
    pb = meshgen.cube_problem(n=2, steps=2)
    e = np.asarray(pb["e"])
    th = np.stack([np.log(e[:, 0]), np.log(e[:, 2]), np.log(e[:, 3])], 1)
    e2 = e.copy()
    e2[:, 0], e2[:, 2], e2[:, 3] = np.exp(th[:, 0]), np.exp(th[:, 1]), np.exp(th[:, 2])
    assert np.allclose(e2, e, rtol=1e-15, atol=0)
    assert e.shape[0] == pb["numel"]  # one material per element
