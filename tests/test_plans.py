"""Region plans: the reference's Euler-tour property test (test/test_euler_tour.jl:7-26)
on both the product's plans and the oracle's restatement, and agreement between them."""
import networksolvers_gb300.models as m
from networksolvers_gb300 import network as pn
from oracle import network as on

GRAPHS = [m.build_tree_graph(3, 3), m.chain_graph(7), m.binary_tree_graph(3), m.chain_plus_ancilla_graph(10)]


def _props(tour, g):
    for j in range(len(tour) - 1):
        assert tour[j][1] == tour[j + 1][0]
    es = set(tour)
    for (u, v) in g.edges:
        assert (u, v) in es and (v, u) in es


def test_euler_tour_reference_properties():
    g = m.build_tree_graph(3, 3)
    for mod in (pn, on):
        G = mod.G(g.vertices, g.edges)
        tour = mod.euler_tour_edges(G, (0, 0))
        _props(tour, g)
        verts = mod.euler_tour_vertices(G, (0, 0))
        for v in g.vertices:
            assert v in verts


def test_plans_agree_with_oracle():
    for g in GRAPHS:
        P, O = pn.G(g.vertices, g.edges), on.G(g.vertices, g.edges)
        assert P.default_root_vertex() == O.default_root_vertex()
        for nsites in (1, 2):
            assert [r for r, _ in pn.euler_sweep(P, nsites)] == [r for r, _ in on.euler_sweep(O, nsites)]
            assert [r for r, _ in pn.post_order_dfs_plan(P, nsites)] == [r for r, _ in on.post_order_dfs_plan(O, nsites)]
            a = pn.tdvp_regions(P, 0.1, {}, 4, nsites)
            b = on.tdvp_regions(O, 0.1, {}, 4, nsites)
            assert [(r, k["updater_kwargs"]["time_step"]) for r, k in a] == [(r, k["updater_kwargs"]["time_step"]) for r, k in b]
        for r1 in ([g.vertices[0]], list(g.vertices)):
            for r2 in ([g.vertices[-1]], [g.vertices[1], g.vertices[2]] if len(g.vertices) > 3 else [g.vertices[1]]):
                assert pn.edge_sequence_between_regions(P, r1, r2) == on.edge_sequence_between_regions(O, r1, r2)


def test_chain_dmrg_plan_shape():
    g = m.chain_graph(20)
    plan = pn.euler_sweep(pn.G(g.vertices, g.edges), 2)
    assert len(plan) == 38
    assert plan[0][0] == [1, 2] and plan[18][0] == [19, 20] and plan[19][0] == [20, 19] and plan[-1][0] == [2, 1]


def test_tdvp_order4_weights():
    w = pn.tdvp_sub_time_steps(4)
    assert abs(sum(w) - 1.0) < 1e-15 and len(w) == 6
