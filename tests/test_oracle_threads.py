"""The oracle's threaded paths (CPU only): per-cell loops on several threads give the serial
cell arrays bit for bit, and the colour-parallel InserterCSC assembly gives the serial
pattern with values equal up to rounding (colour-then-cell order instead of cell order)."""
import numpy as np


def test_cell_threads_change_no_arithmetic(orc):
    rng = np.random.default_rng(3)
    n = 10
    kap = np.exp(rng.standard_normal(n ** 3))
    f = rng.standard_normal((n + 1) ** 3)
    jit = rng.uniform(-0.2, 0.2, ((n + 1) ** 3, 3)) / n
    a = orc.poisson_q1((0, 1) * 3, (n,) * 3, ("boundary",), kappa=kap, fkind=orc.F_NODAL,
                       fdata=f, jitter=jit, assemble=False)
    with orc.cell_threads(4):
        b = orc.poisson_q1((0, 1) * 3, (n,) * 3, ("boundary",), kappa=kap, fkind=orc.F_NODAL,
                           fdata=f, jitter=jit, assemble=False)
    assert np.array_equal(a["cellmats"], b["cellmats"]) and np.array_equal(a["cellvecs"],
                                                                          b["cellvecs"])
    q1 = orc.poisson_q2((0, 1) * 3, (4,) * 3, ("boundary",), fconst=1.0, jitter=jit[:125] * 2.5)
    with orc.cell_threads(4):
        q2 = orc.poisson_q2((0, 1) * 3, (4,) * 3, ("boundary",), fconst=1.0,
                            jitter=jit[:125] * 2.5)
    assert np.array_equal(q1["cellmats"], q2["cellmats"])
    lame = np.exp(rng.standard_normal((6 * 27, 2)))
    e1 = orc.elasticity_p2((0, 1) * 3, (3, 3, 3), lame, assemble=False)
    with orc.cell_threads(4):
        e2 = orc.elasticity_p2((0, 1) * 3, (3, 3, 3), lame, assemble=False)
    assert np.array_equal(e1["cellmats"], e2["cellmats"])


def test_colour_parallel_assembly_matches_serial(orc):
    rng = np.random.default_rng(4)
    for part, tags in (((9, 7, 8), ("boundary",)), ((12, 10), ("tag_7",))):
        nc = int(np.prod(part))
        kap = np.exp(rng.standard_normal(nc))
        f = rng.standard_normal(int(np.prod(np.array(part) + 1)))
        r = orc.poisson_q1((0, 1) * len(part), part, tags, kappa=kap, fkind=orc.F_NODAL, fdata=f)
        col, k = orc.color_cells(r["cell_dofs"], r["nfree"])
        # cells of one colour share no free dof
        for c in range(k):
            ids = r["cell_dofs"][col == c]
            ids = ids[ids > 0]
            assert np.unique(ids).shape[0] == ids.shape[0]
        (cp, rv, zv), b = orc.assemble_colored(r["cell_dofs"], r["cellmats"], r["cellvecs"],
                                               r["nfree"], 4, (col, k))
        c0, r0, z0 = r["csc"]
        assert np.array_equal(cp, c0) and np.array_equal(rv, r0)
        assert np.abs(zv - z0).max() <= 1e-14 * np.abs(z0).max()
        assert np.abs(b - r["b"]).max() <= 1e-14 * np.abs(r["b"]).max()
