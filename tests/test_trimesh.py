"""Rigid triangle-mesh contact (wf_set_contact_trimesh) on the GPU.

The oracle's restatement of CalcContactForces is pinned bit-for-bit to the
reference in tests/test_oracle.py (fixture tet_die_trimesh). Here the FP64
GPU step with a moving die is checked against the oracle on the same inputs:
displacements, contact forces, the reaction history and the die position,
1e-9 relative (the reaction sum runs in a different order on the GPU). The
mixed-precision contact is checked against the FP64 step.
"""
import numpy as np
import pytest

import weldformfem_gb300 as wf
from oracle import orabind as O
from tests import helpers as H
from weldformfem_gb300 import workloads as W

DIE_TET = dict(start=[-0.001, -0.001, 0.002 - 1e-5], end=[0.004, 0.004, 0.0], dens=2, flip=True,
               vel=[0.0, 0.0, -5.0], mu_s=0.1, mu_d=0.08, pf=0.1, end_t=2e-6)
DIE_HEX = dict(start=[-0.0005, -0.0005, 0.004 - 2e-6], end=[0.0045, 0.0045, 0.0], dens=3,
               flip=True, vel=[0.0, 0.0, -4.0], mu_s=0.2, mu_d=0.15, pf=0.3, end_t=1e-5)


def cases():
    t = W.config(1, scale=(3, 3, 4))
    t.perturb = 0.1
    t.bc = "bottom_z"
    h = W.config(0, scale=(4, 4, 4))
    h.perturb = 0.05
    h.seed = W.SEED_BASE + 11
    h.bc = "bottom_z"
    return {"tet": (t, DIE_TET, 300), "hex_hg": (h, DIE_HEX, 400)}


def run(dom, case, die, steps):
    H.setup(dom, case, {"die": die})
    dom.init()
    dom.step(steps) if hasattr(dom, "step") else dom.run(steps)
    return dom


def test_axis_plane_mesh_orientation():
    xyz, tri = W.axis_plane_mesh((0.0, 0.0, 1.0), (2.0, 0.0, 0.0), 2, flip_normals=True)
    assert xyz.shape == (9, 3) and tri.shape == (8, 3) and np.all(xyz[:, 2] == 1.0)
    n = np.cross(xyz[tri[:, 1]] - xyz[tri[:, 0]], xyz[tri[:, 2]] - xyz[tri[:, 0]])
    assert np.all(n[:, 2] < 0)
    _, tri2 = W.axis_plane_mesh((0.0, 0.0, 1.0), (2.0, 0.0, 0.0), 2)
    n2 = np.cross(xyz[tri2[:, 1]] - xyz[tri2[:, 0]], xyz[tri2[:, 2]] - xyz[tri2[:, 0]])
    assert np.all(n2[:, 2] > 0)


def test_add_body_needs_a_first_body():
    o = O.OracleDomain()
    with pytest.raises(RuntimeError):
        o.add_contact_trimesh(np.zeros((3, 3)), np.array([[0, 1, 2]]), [0.0, 0.0, 0.0])


def test_oracle_die_pushes_the_part():
    case, die, steps = cases()["hex_hg"]
    o = run(O.OracleDomain(), case, die, steps)
    r = o.reaction()
    assert r.shape == (steps,) and r.max() > 0 and np.all(np.isfinite(o.node_vec("u")))
    top = case.top_nodes()
    assert o.node_vec("u")[top, 2].mean() < 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tet", "hex_hg"])
def test_trimesh_contact_matches_oracle(name):
    case, die, steps = cases()[name]
    o = run(O.OracleDomain(), case, die, steps)
    d = wf.Domain(wf.WF_FP64)
    H.setup(d, case, {"die": die})
    d.init()
    d.run(steps)
    assert H.rel_err(d.node_vec("u"), o.node_vec("u")) <= 1e-9
    assert H.rel_err(d.node_vec("contforce"), o.node_vec("contforce")) <= 1e-9
    assert H.rel_err(d.reaction(), o.reaction()) <= 1e-9
    np.testing.assert_allclose(d.trimesh_nodes(), o.trimesh_nodes(), rtol=1e-12, atol=0)
    assert o.reaction().max() > 0


DIE_BOTTOM = dict(start=[-0.001, -0.001, 1e-5], end=[0.004, 0.004, 0.0], dens=3, flip=False,
                  vel=[0.0, 0.0, 2.0])


@pytest.mark.gpu
def test_two_rigid_bodies_match_oracle():
    """Top die (body 0) and a rising bottom plate (body 1, wf_add_contact_trimesh)
    squeezing a block held only by x/y symmetry planes: only the top die's
    contacts feed the reaction."""
    case = W.config(1, scale=(3, 3, 4))
    case.perturb = 0.1
    case.seed = W.SEED_BASE + 13
    case.bc = "sym_xy"
    extra = {"die": DIE_TET, "die2": DIE_BOTTOM}
    steps = 300
    o = O.OracleDomain()
    H.setup(o, case, extra)
    o.init()
    o.step(steps)
    d = wf.Domain(wf.WF_FP64)
    H.setup(d, case, extra)
    d.init()
    d.run(steps)
    assert H.rel_err(d.node_vec("u"), o.node_vec("u")) <= 1e-9
    cf = d.node_vec("contforce")
    assert H.rel_err(cf, o.node_vec("contforce")) <= 1e-9
    assert H.rel_err(d.reaction(), o.reaction()) <= 1e-9
    np.testing.assert_allclose(d.trimesh_nodes(), o.trimesh_nodes(), rtol=1e-12, atol=0)
    x0 = case.coords()
    assert cf[x0[:, 2] < 1e-12, 2].max() > 0      # the plate pushes up
    assert d.trimesh_nodes().shape == (9 + 16, 3)


def off_grid(die, dx=1.1e-4, dy=7e-5):
    """The die shifted so that no part node lies on a die edge. The
    reference's inside test (crit < 0 rejects) decides a node that lies exactly
    on an edge shared by two triangles by the sign of a rounding error: in
    either precision it may find both triangles or neither, so runs that differ
    by rounding are compared on dies whose edges avoid the part's nodes."""
    d = dict(die)
    d["start"] = [die["start"][0] + dx, die["start"][1] + dy, die["start"][2]]
    return d


def mixed_vs_fp64(case, extra, steps, mode=0):
    out = []
    for prec in (wf.WF_FP64, wf.WF_MIXED):
        d = wf.Domain(prec)
        H.setup(d, case, extra)
        if prec == wf.WF_MIXED:
            d.set_step_mode(mode)
        d.init()
        d.run(steps)
        out.append(d)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tet", "hex_hg"])
def test_mixed_trimesh_contact_against_fp64(name):
    """FP32 contact (coordinates relative to the part's centre, die kept in
    FP64 and copied to FP32 after every move) against the FP64 step."""
    case, die, steps = cases()[name]
    f, m = mixed_vs_fp64(case, {"die": off_grid(die)}, steps)
    eu = H.rel_err(m.node_vec("u"), f.node_vec("u"))
    er = H.rel_err(m.reaction(), f.reaction())
    print(f"{name}: mixed vs FP64 displacement {eu:.2e}, reaction {er:.2e}")
    assert eu <= 1e-4 and er <= 1e-3
    np.testing.assert_allclose(m.trimesh_nodes(), f.trimesh_nodes(), rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_mixed_two_bodies_cluster_run_is_bitwise_the_graph_run():
    """Two rigid bodies in mixed precision: the single-cluster run (die moved
    by block 0) and the per-phase kernels give the same state bit for bit."""
    case = W.config(1, scale=(3, 3, 4))
    case.perturb = 0.1
    case.seed = W.SEED_BASE + 13
    case.bc = "sym_xy"
    extra = {"die": off_grid(DIE_TET), "die2": off_grid(DIE_BOTTOM, 1.3e-4, -1.9e-4)}
    runs = []
    for mode in (1, 2):
        d = wf.Domain(wf.WF_MIXED)
        H.setup(d, case, extra)
        d.set_step_mode(mode)
        d.init()
        assert d.step_mode()[0] == mode
        d.run(150)
        d.run(150)
        runs.append(d)
    a, b = runs
    for f in ("u", "v", "contforce"):
        np.testing.assert_array_equal(b.node_vec(f), a.node_vec(f), err_msg=f)
    np.testing.assert_array_equal(b.trimesh_nodes(), a.trimesh_nodes())
    assert H.rel_err(b.reaction(), a.reaction()) <= 1e-12
    # against FP64: the dies carry Coulomb friction, whose sliding direction
    # -v_t / |v_t| is set by rounding where the tangential velocity is near
    # zero, so the bound is on the RMS displacement error and the reaction
    # history (as for the other frictional cases); measured: 4.4e-5 and
    # 3.7e-5 after 300 steps, 5e-6 for both after 100 and 200 steps
    f, _ = mixed_vs_fp64(case, extra, 300)
    u, uf = a.node_vec("u"), f.node_vec("u")
    assert np.sqrt(np.mean((u - uf) ** 2)) / np.sqrt(np.mean(uf ** 2)) <= 1e-3
    assert H.rel_err(a.reaction(), f.reaction()) <= 1e-3
