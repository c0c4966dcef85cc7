"""CPU tests of the oracle itself: pinned against the reference's own KD tree (golden fixtures and, where the
reference checkout exists, live), closed-form assembly properties, CG residuals and the expression language."""
import numpy as np
import pytest

import oracle
from navier_stokes_fem_gb300 import mesh as M
from tests._meshes import golden_mesh, rel

TAGS = ["mesh_small", "cavity32", "perturbed12"]


@pytest.mark.parametrize("tag", TAGS)
def test_oracle_tree_matches_reference_fixture(golden, tag):
    m = golden_mesh(golden, tag)
    o = oracle.Oracle(m, 0.01, 0.01) if m.u_dirichlet else _oracle_no_bc(m)
    e, xi, eta, nn = o.locate(golden[f"{tag}/points"])
    assert np.array_equal(e, golden[f"{tag}/elem"])
    assert np.array_equal(xi.view(np.uint32), golden[f"{tag}/xi"].view(np.uint32))
    assert np.array_equal(eta.view(np.uint32), golden[f"{tag}/eta"].view(np.uint32))
    assert np.array_equal(nn, golden[f"{tag}/nearest"])
    assert (e < 0).sum() > 100 and (e >= 0).sum() > 1000


def _oracle_no_bc(m, nu=0.01, dt=0.01):
    return oracle.Oracle(m, nu, dt)


def test_reference_grid_bbox_quirk(golden):
    # BBox2D::expand keeps the LAST node as the max corner (gpu_cpu_shared/misc_common.cuh:59-65)
    bb = golden["cavity32/bbox"]
    last = golden["cavity32/nodes"][-1]
    assert bb[0] == 0 and bb[1] == 0 and bb[2] == last[0] and bb[3] == last[1]
    assert bb[2] < 1.0


@pytest.mark.skipif(not oracle.ref_available(), reason="reference checkout not compiled here")
def test_oracle_tree_matches_reference_live():
    m = M.channel_with_obstacle(64, 16)
    rng = np.random.default_rng(5)
    pts = np.concatenate([rng.uniform([-0.1, -0.1], [4.1, 1.1], size=(20000, 2)), m.nodes]).astype(np.float32)
    a = oracle.Oracle(m, 1e-3, 2e-3).locate(pts)
    b = oracle.ReferenceTree(m).locate(pts)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_tree_depth_rule():
    # maxDepth = min(29, round(8 + 1.3 ln T)) (cpp/kd_tree_builder.cpp:87)
    for n in (4, 16, 32):
        m = M.cavity(n)
        o = oracle.Oracle(m, 0.01, 0.01)
        _, _, depth = o.tree_size()
        assert depth == min(29, int(round(8 + 1.3 * np.log(np.float32(2 * n * n)))))


@pytest.mark.parametrize("n", [4, 16])
def test_mass_and_stiffness_closed_forms(n):
    m = M.cavity(n)
    m.u_dirichlet, m.p_dirichlet = [], []            # no elimination: the raw operators
    o = oracle.Oracle(m, 0.5, 0.1)
    Mm = o.scipy_matrix("velocity_mass")
    D = o.scipy_matrix("diffusion")
    K = o.scipy_matrix("pressure_stiffness")
    B = o.scipy_matrix("velocity_divergence")
    G = o.scipy_matrix("pressure_divergence")
    one_v, one_p = np.ones(m.n_nodes), np.ones(m.n_pressure)
    assert abs(Mm.sum() - 1.0) < 1e-13                       # sum of all mass entries = area
    # P2: vertex shape functions integrate to 0, midside ones to |T|/3
    row = Mm @ one_v
    assert np.abs(row[: m.n_pressure]).max() < 1e-14
    assert np.allclose(row[m.n_pressure:].sum(), 1.0, atol=1e-13)
    assert np.abs(K @ one_p).max() < 1e-12                  # stiffness annihilates constants
    assert np.abs(D @ one_v - row).max() < 1e-12            # diffusion = M + dt*nu*K
    assert np.abs(B @ np.ones(2 * m.n_nodes)).max() < 1e-9  # div of a constant field
    assert np.abs(G @ one_p).max() < 1e-12                  # grad of a constant pressure
    assert abs(Mm - Mm.T).max() < 1e-15 and abs(K - K.T).max() < 1e-15


def test_cavity_pattern_counts():
    # nnz of the P2 pattern 46n^2+16n+1 and of the P1 pattern 7n^2+6n+1 on the diagonal-split cavity
    for n in (4, 32):
        m = M.cavity(n)
        m.u_dirichlet, m.p_dirichlet = [], []
        o = oracle.Oracle(m, 0.01, 0.01)
        assert o.matrix("velocity_mass")[1].size == 46 * n * n + 16 * n + 1
        assert o.matrix("pressure_stiffness")[1].size == 7 * n * n + 6 * n + 1


def test_manufactured_poisson_solutions_converge_at_the_element_orders():
    """-lap u = f on the unit square with u = sin(pi x) sin(pi y), u = 0 on the boundary, assembled by the oracle:
    P2 (stiffness = (diffusion - mass) / (dt nu), load = M f) and P1 (the pressure stiffness, load = the P1
    vertex rows of M f summed from the P2 mass, which integrates f against the P1 hat functions exactly for P2
    data).  The nodal errors fall with h at the elements' orders: h^2 for P1 and, at the nodes of this uniform
    mesh, h^4 for P2 (superconvergent; h^3 in general)."""
    import scipy.sparse.linalg as spla

    err2, err1 = [], []
    for n in (8, 16, 32):
        m = M.cavity(n)
        m.u_dirichlet, m.p_dirichlet = [], []
        o = oracle.Oracle(m, 1.0, 1.0)                      # diffusion = M + 1 * 1 * K
        Mm, D, K1 = (o.scipy_matrix(k).tocsr() for k in ("velocity_mass", "diffusion", "pressure_stiffness"))
        K2 = (D - Mm).tocsr()
        xy = m.nodes.astype(np.float64)
        u = np.sin(np.pi * xy[:, 0]) * np.sin(np.pi * xy[:, 1])
        on_b = (np.abs(xy[:, 0]) < 1e-12) | (np.abs(xy[:, 0] - 1) < 1e-12) | \
               (np.abs(xy[:, 1]) < 1e-12) | (np.abs(xy[:, 1] - 1) < 1e-12)
        b2 = Mm @ (2 * np.pi ** 2 * u)
        free = np.flatnonzero(~on_b)
        uh = np.zeros_like(u)
        uh[free] = spla.spsolve(K2[free][:, free].tocsc(), b2[free])
        err2.append(np.abs(uh - u).max())
        # P1 on the vertices: the P1 hat of vertex i is its P2 vertex function plus half of each adjacent
        # midside function, so the P1 load is (M f)_i + half the load of the midside nodes around it
        P = m.n_pressure
        el = m.elements
        b1 = b2[:P].copy()
        mids = {}   # midside node -> its edge's vertices (element node order [v0, v1, v2, m12, m02, m01])
        for e in el:
            for (i, j, k) in ((e[1], e[2], e[3]), (e[0], e[2], e[4]), (e[0], e[1], e[5])):
                mids[int(k)] = (int(i), int(j))
        for k, (i, j) in mids.items():
            b1[i] += 0.5 * b2[k]
            b1[j] += 0.5 * b2[k]
        free1 = np.flatnonzero(~on_b[:P])
        ph = np.zeros(P)
        ph[free1] = spla.spsolve(K1[free1][:, free1].tocsc(), b1[free1])
        err1.append(np.abs(ph - u[:P]).max())
    r2 = np.log2(np.array(err2[:-1]) / np.array(err2[1:]))
    r1 = np.log2(np.array(err1[:-1]) / np.array(err1[1:]))
    assert err2[-1] < 1e-6 and (r2 > 3.5).all(), (err2, r2)   # measured 3.88, 3.96
    assert err1[-1] < 1e-3 and (r1 > 1.9).all(), (err1, r1)   # measured 2.00, 2.00


def test_divergence_and_gradient_scalings_on_linear_fields():
    """The step's operators carry the reference's scalings (include/assembly.h:1302-1475): B = -(1/dt) div and
    Bp = -dt grad.  With the shape functions summing to one, sum_i (B (x, y))_i = -(1/dt) * 2 * area and
    sum_j (Bp x)_j = -dt * area in the x block and 0 in the y block (unit square)."""
    m = M.cavity(8)
    m.u_dirichlet, m.p_dirichlet = [], []
    dt = 0.1
    o = oracle.Oracle(m, 0.5, dt)
    B, G = o.scipy_matrix("velocity_divergence"), o.scipy_matrix("pressure_divergence")
    xy = m.nodes.astype(np.float64)
    nv, P = m.n_nodes, m.n_pressure
    assert B.shape == (P, 2 * nv) and G.shape == (2 * nv, P)      # y block at column / row offset Nv
    assert abs((B @ np.concatenate([xy[:, 0], xy[:, 1]])).sum() + 2 / dt) < 1e-11
    assert abs((B @ np.concatenate([xy[:, 0], 0 * xy[:, 1]])).sum() + 1 / dt) < 1e-11
    g = G @ xy[:P, 0]
    assert abs(g[:nv].sum() + dt) < 1e-14 and abs(g[nv:].sum()) < 1e-14


def test_uniform_flow_is_a_steady_state_of_the_step():
    """u = (1, 0) with the same Dirichlet data on every wall: advection moves a constant to itself, the diffusion
    solve returns it (the stiffness annihilates constants), its divergence is zero so the pressure stays 0 and the
    projection changes nothing.  Three operator-split steps keep it to rounding."""
    m = M.cavity(8)
    m.u_dirichlet = [(g[0], "1", "0") for g in m.u_dirichlet]
    o = oracle.Oracle(m, 0.01, 0.05)
    nv = m.n_nodes
    o.set_fields(np.concatenate([np.ones(nv), np.zeros(nv)]), np.zeros(m.n_pressure))
    st, _ = o.step(3)
    uv, p = o.fields()
    assert st == 0
    assert np.abs(uv[:nv] - 1).max() < 1e-12 and np.abs(uv[nv:]).max() < 1e-12 and np.abs(p).max() < 1e-12


def test_uniform_flow_is_a_steady_state_of_the_explicit_scheme():
    """The explicit-convection scheme (the reference's NavierStokesAssembly::solve): the convection of a constant
    velocity is zero (its nodal values are equal, so u_h . grad u_h vanishes) and the stiffness annihilates it, so the
    tentative increment is zero; the divergence is zero, the pressure stays 0 and the correction is zero."""
    m = M.cavity(8)
    m.u_dirichlet = [(g[0], "1", "0.5") for g in m.u_dirichlet]
    o = oracle.Oracle(m, 0.01, 0.02)
    o.set_scheme("explicit_convection")
    nv = m.n_nodes
    o.set_fields(np.concatenate([np.ones(nv), np.full(nv, 0.5)]), np.zeros(m.n_pressure))
    st, _ = o.step(3)
    uv, p = o.fields()
    assert st == 0
    assert np.abs(uv[:nv] - 1).max() < 1e-12 and np.abs(uv[nv:] - 0.5).max() < 1e-12 and np.abs(p).max() < 1e-12


def test_advection_reproduces_quadratic_fields_exactly():
    """Semi-Lagrangian self-advection of u = y^2, v = x^2 (both in the P2 space): the departure point of node x is
    x - dt (u, v), and P2 interpolation there reproduces the quadratics, so the new fields are (y - dt x^2)^2 and
    (x - dt y^2)^2 at every node whose departure point stays inside the square, up to the rounding of the float
    departure points and barycentric coordinates."""
    dt = 0.05
    m = M.cavity(16)
    o = oracle.Oracle(m, 0.01, dt)
    xy = m.nodes.astype(np.float64)
    u, v = xy[:, 1] ** 2, xy[:, 0] ** 2
    un, vn = o.advect(u, v)
    dx, dy = xy[:, 0] - dt * u, xy[:, 1] - dt * v
    inside = (dx > 1e-3) & (dx < 1 - 1e-3) & (dy > 1e-3) & (dy < 1 - 1e-3)
    assert inside.sum() > 0.8 * m.n_nodes
    assert np.abs(un[inside] - dy[inside] ** 2).max() < 1e-7   # measured 2.4e-8
    assert np.abs(vn[inside] - dx[inside] ** 2).max() < 1e-7


def test_dirichlet_elimination_structure():
    m = M.cavity(8)
    o = oracle.Oracle(m, 0.01, 0.01)
    D = o.scipy_matrix("diffusion").tocsr()
    bc = np.unique(np.concatenate([g[0] for g in m.u_dirichlet]))
    for r in bc[:20]:
        row = D.getrow(r)
        assert row.nnz == 1 and row.indices[0] == r and row.data[0] == 1.0
    free = np.setdiff1d(np.arange(m.n_nodes), bc)
    assert abs(D[free][:, bc]).max() == 0
    W = o.scipy_matrix("velocity_dirichlet_weights")      # transposed storage: row = Dirichlet node
    assert set(np.unique(W.tocoo().row)).issubset(set(bc))
    # the values: the free block is the raw operator's, and W holds the raw couplings of the free rows to the
    # Dirichlet columns, so D_e x = b_e with b_e[free] = b[free] - (W^T g)[free] is the raw system with x[bc] = g
    m2 = M.cavity(8)
    m2.u_dirichlet, m2.p_dirichlet = [], []
    Dr = oracle.Oracle(m2, 0.01, 0.01).scipy_matrix("diffusion").tocsr()
    W = W.tocsr()
    assert abs(D[free][:, free] - Dr[free][:, free]).max() == 0
    assert abs(W[bc][:, free] - Dr[free][:, bc].T).max() == 0


def test_cg_oracle_relative_residual():
    m = M.cavity(16)
    o = oracle.Oracle(m, 0.01, 0.01)
    A = o.scipy_matrix("pressure_stiffness")
    rng = np.random.default_rng(3)
    b = rng.standard_normal(A.shape[0])
    x, st, it, rr = o.cg("pressure_stiffness", b, np.zeros_like(b))
    assert st == 0 and it > 10
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) < 1.5e-8
    # already converged initial guess: zero iterations, x = x0
    x2, st2, it2, _ = o.cg("pressure_stiffness", b, x)
    assert st2 == 0 and it2 == 0 and np.array_equal(x2, x)


def test_oracle_fp32_tracks_fp64():
    m = M.cavity(16)
    a, b = oracle.Oracle(m, 0.01, 0.01), oracle.Oracle(m, 0.01, 0.01, real_bits=32)
    a.step(5)
    b.step(5)
    assert rel(b.fields()[0], a.fields()[0]) < 1e-4


@pytest.mark.parametrize("expr,x,y,value", [
    ("4*1.5*y*(0.41-y)/(0.41*0.41)", 0.0, 0.205, 1.5), ("-2^2", 0, 0, -4.0), ("2^-1", 0, 0, 0.5),
    ("2^3^2", 0, 0, 64.0), ("sin(Pi/2)+cos(0)*E", 0, 0, 1 + np.e), ("1-x-y*3/2", 0.25, 0.5, 0.0),
    ("-(x+1)*-2", 1.0, 0, 4.0), ("4*y*(1-y)", 0, 0.5, 1.0), ("0", 3, 4, 0.0), ("1e-3*x", 2, 0, 2e-3),
])
def test_expression_known_answers(expr, x, y, value):
    import navier_stokes_fem_gb300 as nsf

    assert oracle.evaluate_expression(expr, {"x": x, "y": y}) == pytest.approx(value, abs=1e-15)
    assert nsf.evaluate_expression(expr, x, y) == pytest.approx(value, abs=1e-15)


TIMED_EXPRESSIONS = ["4*1.5*y*(0.41-y)/(0.41*0.41)*sin(Pi*t/8)", "-x^2^-1+t", "2^-t*cos(x-y*t)/3", "1-t/2*-x",
                     "E^(t*x)-Pi*-(y)", "(x+y)*(x-y)^2/(1+t)", "sin(cos(t))*-3^2", "0.15*t-x/y/t"]


@pytest.mark.parametrize("expr", TIMED_EXPRESSIONS)
def test_time_dependent_expression_programs(expr):
    """The postfix program that nsf_sim_set_bc_expressions compiles for the device, run op for op on the host
    (nsf_eval_expression_t), gives the oracle's tree-walk value bit for bit: precedence, associativity and unary
    minus survive the compilation."""
    import navier_stokes_fem_gb300 as nsf

    for x, y, t in [(0.3, 0.2, 0.05), (1.0, 0.37, 2.5), (0.7, 0.1, 1e-3)]:
        assert nsf.evaluate_expression(expr, x, y, t) == oracle.evaluate_expression(expr, {"x": x, "y": y, "t": t})


def _expression_fixture():
    import json
    import os

    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_expressions.json")) as f:
        return json.load(f)


def test_expressions_match_reference_evaluator():
    """The restated expression language (oracle) and the product's host evaluator, both in double at the points'
    float coordinates, against the reference's own Expression::evaluate in float (tests/golden/ref_expressions.json,
    written by make_expression_golden.py from cpp/expression.cpp): within 8 float ulps of the value (the
    reference rounds every operation to float).  Texts the reference rejects are rejected by both.  Two texts the
    reference cannot be run on in-process ("(1+2" ends it in an assert, "1+*" does not terminate) are covered by
    test_expression_errors: both evaluators here return an error for them."""
    import navier_stokes_fem_gb300 as nsf

    g = _expression_fixture()
    pts = [tuple(float(np.float32(v)) for v in p) for p in g["points"]]
    assert len(g["values"]) >= 20
    for expr, want in g["values"].items():
        for (x, y, t), w in zip(pts, want):
            got = oracle.evaluate_expression(expr, {"x": x, "y": y, "t": t})
            assert abs(got - w) <= 8 * 2.0 ** -24 * abs(w), (expr, x, y, t, got, w)
            assert nsf.evaluate_expression(expr, x, y, t) == got
    for bad in g["rejected"]:
        with pytest.raises(Exception):
            oracle.evaluate_expression(bad, {"x": 0.0, "y": 0.0, "t": 0.0})
        with pytest.raises(Exception):
            nsf.evaluate_expression(bad, 0.0, 0.0, 0.0)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference checkout not compiled here")
def test_expressions_match_reference_evaluator_live():
    g = _expression_fixture()
    for expr, want in g["values"].items():
        assert [oracle.ref_evaluate_expression(expr, *p) for p in g["points"]] == want, expr
    for bad, where in g["rejected"].items():
        with pytest.raises(ValueError, match=f"\\({where}\\)"):
            oracle.ref_evaluate_expression(bad, *g["points"][0])


def _float_dirichlet_shift(golden, float_values):
    """Relative change of the fields of 20 oracle steps on mesh_small (driven to 1e-13) when its Dirichlet values
    are replaced by float_values(mesh, gu, gv, gp)."""
    m = golden_mesh(golden, "mesh_small")
    a, b = oracle.Oracle(m, 0.001, 0.01), oracle.Oracle(m, 0.001, 0.01)
    _, gu, gv, _, gp = oracle.bc_occurrences(m)
    fu, fv, fp = (np.ascontiguousarray(v, np.float64) for v in float_values(m, gu, gv, gp))
    assert 0 < np.abs(fu - gu).max() < 1e-6
    oracle.lib().orc_set_bc(b._h, fu, fv, fp)
    for o in (a, b):
        o.set_tolerance(1e-13)
        assert o.step(20)[0] == 0
    (ua, pa), (ub, pb) = a.fields(), b.fields()
    a.close()
    b.close()
    return rel(ub, ua), rel(pb, pa)


def test_float_dirichlet_values_shift_the_fields_below_the_field_tolerance(golden):
    """Deviation kept on purpose: the reference evaluates the Dirichlet expressions in float every step
    (cpp/grid.cpp:80-94, include/assembly.h:1559-1579), this library once in double.  With the double values rounded
    to float, the fields of 20 steps on mesh_small move by about 1e-8 (velocity) and 7e-8 (pressure) relative,
    far below the 1e-6 field tolerance of the GPU parity tests."""
    duv, dp = _float_dirichlet_shift(golden, lambda m, gu, gv, gp: (np.float32(gu), np.float32(gv), np.float32(gp)))
    assert 0 < duv < 1e-7 and dp < 1e-6, (duv, dp)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference checkout not compiled here")
def test_float_dirichlet_values_shift_the_fields_below_the_field_tolerance_live(golden):
    """The same with the values the reference's own Expression::evaluate gives in float at every occurrence
    (measured: 4.9e-8 velocity, 1.4e-7 pressure)."""
    def ref_values(m, gu, gv, gp):
        out = ([], [], [])
        for nodes, ue, ve in m.u_dirichlet:
            for nd in nodes:
                x, y = float(m.nodes[nd, 0]), float(m.nodes[nd, 1])
                out[0].append(oracle.ref_evaluate_expression(ue, x, y))
                out[1].append(oracle.ref_evaluate_expression(ve, x, y))
        for nodes, pe in m.p_dirichlet:
            for nd in nodes:
                out[2].append(oracle.ref_evaluate_expression(pe, float(m.nodes[nd, 0]), float(m.nodes[nd, 1])))
        return out

    duv, dp = _float_dirichlet_shift(golden, ref_values)
    assert 0 < duv < 1e-6 and dp < 1e-6, (duv, dp)


def test_oracle_time_dependent_stepping_known_answer():
    """A lid written as "1 + 0*t" goes through the oracle's per-step re-evaluation at t = k dt and must give the
    constant lid's fields bit for bit (one thread: the oracle's parallel reductions are not ordered); a lid that
    changes with t must not."""
    fields = {}
    prev = oracle.max_threads()
    oracle.set_threads(1)
    try:
        for lid in ("1", "1+0*t", "1+t"):
            o = oracle.Oracle(M.cavity(8, lid_u=lid), 0.01, 0.05)
            assert o.timed == ("t" in lid)
            st, _ = o.step(4)
            assert st == 0
            fields[lid] = o.fields()
            o.close()
    finally:
        oracle.set_threads(prev)
    assert all(np.array_equal(a, b) for a, b in zip(fields["1"], fields["1+0*t"]))
    assert not np.array_equal(fields["1"][0], fields["1+t"][0])


@pytest.mark.parametrize("bad", ["z+1", "(1+2", "sin 3", "1+*", "x$"])
def test_expression_errors(bad):
    import navier_stokes_fem_gb300 as nsf

    with pytest.raises(Exception):
        nsf.evaluate_expression(bad, 0.0, 0.0)
    with pytest.raises(Exception):
        oracle.evaluate_expression(bad, {"x": 0.0, "y": 0.0})


def test_mesh_generators():
    c = M.cavity(32)
    assert (c.n_elements, c.n_nodes, c.n_pressure) == (2048, 4225, 1089)
    ch = M.channel_with_obstacle(1024, 256)
    assert ch.n_elements == 2 * (1024 * 256 - 50 * 50)
    assert ch.n_nodes == 2049 * 513 - 99 * 99
    for m in (c, ch):
        v = m.nodes[m.elements[:, :3]].astype(np.float64)
        area = (v[:, 1, 0] - v[:, 0, 0]) * (v[:, 2, 1] - v[:, 0, 1]) - (v[:, 1, 1] - v[:, 0, 1]) * (v[:, 2, 0] - v[:, 0, 0])
        assert (area > 0).all()                                # counter-clockwise
        allbc = np.concatenate([g[0] for g in m.u_dirichlet])
        assert len(allbc) == len(np.unique(allbc))              # each boundary node in one group
        assert m.elements[:, :3].max() < m.n_pressure <= m.elements[:, 3:].min()


def test_mesh_json_roundtrip(tmp_path):
    m = M.cavity(4)
    p = tmp_path / "m.json"
    M.write_mesh_json(m, str(p))
    r = M.read_mesh_json(str(p))
    assert np.array_equal(r.nodes, m.nodes) and np.array_equal(r.elements, m.elements)
    assert [g[1:] for g in r.u_dirichlet] == [g[1:] for g in m.u_dirichlet]
    s = tmp_path / "scene.json"
    M.write_scene_json(str(s), "m.json", 1.0, 0.01, 0.01)
    sc = M.read_scene_json(str(s))
    assert sc["mesh_path"] == str(p)


@pytest.mark.parametrize("n", [256, 1024])
def test_oracle_port_tree_matches_large_reference_fixture(n):
    """The oracle's restatement of the reference tree against the reference's own (int-offset) tree on every
    departure point of the 256^2 and 1024^2 cavities (digests over all points written from the reference)."""
    import json
    import os

    from tests._meshes import departure_points, lookup_digests, nearest_ties_ok

    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_kdtree_lookup_large.npz"))
    m = M.cavity(n)
    pts = departure_points(m)
    t = oracle.PortTree(m)
    e, xi, eta, nn = t.locate(pts)
    stats = t.stats()
    t.close()
    rec = json.loads(str(g[f"n{n}/record"][0]))
    assert stats["leaf_entries"] == rec["leaf_entries"] and stats["max_depth"] == rec["max_depth"]
    assert lookup_digests(e, xi, eta) == [str(d) for d in g[f"n{n}/digests"]]
    outside = g[f"n{n}/outside"]
    assert np.array_equal(np.nonzero(e < 0)[0], outside)
    nearest_ties_ok(m, pts[outside], nn[outside], g[f"n{n}/outside_nearest"])


def _assembly_fixture():
    import os

    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_local_matrices.npz"))


def test_local_matrices_match_reference_element_code():
    """The oracle's local element matrices against the reference's own element code (shape functions, quadrature,
    Jacobian and local functors of include/assembly.h compiled from its lines): bit-identical in the reference's
    float arithmetic, and the FP64 oracle within float rounding of them (the stiffness cancels, so 1e-5 of the
    largest entry)."""
    g = _assembly_fixture()
    v = g["vertices"]
    o32 = oracle.local_matrices(v, 32)
    o64 = oracle.local_matrices(v, 64)
    for k in oracle.LOCAL_MATRIX_SHAPES:
        ref = g[k].astype(np.float64)
        assert np.array_equal(o32[k], ref), k
        scale = np.abs(o64[k]).max(axis=(1, 2), keepdims=True)
        assert (np.abs(o64[k] - ref) <= 1e-5 * scale).all(), k


def test_local_convection_matches_reference_element_code():
    """The oracle's local convection matrices (the explicit-convection scheme's C(u)) against the reference's own
    convection functor of assembleConvectionMatrix (include/assembly.h:1584-1622, compiled from its lines) on the
    fixture's 996 triangles with seeded nodal velocities: bit-identical in the reference's float arithmetic, the FP64
    oracle within float rounding.  Known answers in FP64: the rows sum to zero (the shape-function gradients sum to
    zero), and for a constant velocity (a, b) and a linear field c x + d y the product is (a c + b d) times the local
    mass row sums (the integrand is psi_i times a constant, integrated exactly)."""
    g = _assembly_fixture()
    v, vel = g["vertices"], g["velocities"]
    o32 = oracle.local_convection(v, vel, 32)
    o64 = oracle.local_convection(v, vel, 64)
    ref = g["convection"].astype(np.float64)
    assert np.array_equal(o32, ref)
    scale = np.abs(o64).max(axis=(1, 2), keepdims=True)
    assert (np.abs(o64 - ref) <= 1e-5 * scale).all()
    assert (np.abs(o64.sum(axis=2)) <= 1e-12 * scale[:, :, 0]).all()
    # constant velocity, linear field
    a, b_, c, d = 0.7, -1.3, 2.0, 0.5
    n = len(v)
    const = np.concatenate([np.full((n, 6), a), np.full((n, 6), b_)], axis=1)
    C = oracle.local_convection(v, const, 64)
    xy = v.astype(np.float64).reshape(n, 3, 2)
    mid = np.stack([(xy[:, 1] + xy[:, 2]) / 2, (xy[:, 0] + xy[:, 2]) / 2, (xy[:, 0] + xy[:, 1]) / 2], axis=1)
    nodes = np.concatenate([xy, mid], axis=1)                        # element node order v0 v1 v2 m12 m02 m01
    phi = c * nodes[:, :, 0] + d * nodes[:, :, 1]
    mass = oracle.local_matrices(v, 64)["mass"]
    want = (a * c + b_ * d) * mass.sum(axis=2)
    got = np.einsum("nij,nj->ni", C, phi)
    assert np.abs(got - want).max() <= 1e-12 * max(1.0, np.abs(want).max())


@pytest.mark.skipif(not oracle.ref_assembly_available(), reason="reference element code not compiled here")
def test_local_convection_matches_reference_element_code_live():
    g = _assembly_fixture()
    live = oracle.ref_local_convection(g["vertices"], g["velocities"])
    assert np.array_equal(live, g["convection"])


@pytest.mark.skipif(not oracle.ref_assembly_available(), reason="reference element code not compiled here")
def test_local_matrices_match_reference_element_code_live():
    g = _assembly_fixture()
    v = g["vertices"]
    live = oracle.ref_local_matrices(v)
    for k in oracle.LOCAL_MATRIX_SHAPES:
        assert np.array_equal(live[k], g[k]), k
