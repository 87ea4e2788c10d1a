"""Pattern and graph sets shared by the tests."""
import json
import os

import fsgc

HERE = os.path.dirname(os.path.abspath(__file__))

# the workload patterns (ER triangle + 2 fringes, and the eight RMAT patterns): (n, undirected edges)
WORKLOAD = {
    "er_triangle_2fringes": (5, [(0, 1), (1, 2), (0, 2), (0, 3), (1, 4)]),
    "wedge_1_on_centre": (4, [(0, 1), (0, 2), (0, 3)]),
    "wedge_2_on_centre": (5, [(0, 1), (0, 2), (0, 3), (0, 4)]),
    "wedge_4_on_centre": (7, [(0, 1), (0, 2), (0, 3), (0, 4), (0, 5), (0, 6)]),
    "wedge_1_on_each_end": (5, [(0, 1), (0, 2), (1, 3), (2, 4)]),
    "triangle_3_on_one": (6, [(0, 1), (1, 2), (0, 2), (0, 3), (0, 4), (0, 5)]),
    "4cycle_opposite": (6, [(0, 1), (1, 2), (2, 3), (3, 0), (0, 4), (2, 5)]),
    "4clique_3_distinct": (7, [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3), (0, 4), (1, 5), (2, 6)]),
    "edge_5_5": (12, [(0, 1)] + [(0, i) for i in range(2, 7)] + [(1, i) for i in range(7, 12)]),
}

CONFIG2 = ["wedge_1_on_centre", "wedge_2_on_centre", "wedge_4_on_centre", "wedge_1_on_each_end",
           "triangle_3_on_one", "4cycle_opposite", "4clique_3_distinct", "edge_5_5"]

# extra shapes that reach every kernel variant
EXTRA = {
    "triangle": (3, [(0, 1), (1, 2), (0, 2)]),
    "tailed_triangle_1": (4, [(0, 1), (1, 2), (0, 2), (0, 3)]),
    "4clique": (4, [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]),
    "tailed_4clique_2": (6, [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3), (0, 4), (0, 5)]),
    "5cycle": (5, [(0, 1), (1, 2), (2, 3), (3, 4), (4, 0)]),
    "5cycle_chord_fringe": (6, [(0, 1), (1, 2), (2, 3), (3, 4), (4, 0), (5, 0), (5, 2)]),
    "house": (5, [(0, 1), (0, 3), (0, 4), (1, 2), (1, 4), (2, 3)]),
    "wedge_centre_and_ends": (6, [(0, 1), (0, 2), (0, 3), (1, 4), (2, 5)]),
    "triangle_mixed": (7, [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (1, 4), (2, 5), (2, 6)]),
    "edge_3_2_shared1": (8, [(0, 1), (0, 2), (0, 3), (0, 4), (1, 5), (1, 6), (0, 7), (1, 7)]),
    "star_12": (13, [(0, i) for i in range(1, 13)]),
    "edge_8_3": (13, [(0, 1)] + [(0, i) for i in range(2, 10)] + [(1, i) for i in range(10, 13)]),
}


def golden_cases(kind=None):
    with open(os.path.join(HERE, "golden", "matching_orders.json")) as f:
        cases = json.load(f)["cases"]
    return [c for c in cases if kind is None or c["kind"] == kind]


def mo_of(n, edges):
    return fsgc.preprocess(n, edges)


def complete_graph(n):
    pairs = [(i, j) for i in range(n) for j in range(i + 1, n)]
    return fsgc.csr_from_edges(n, pairs)


def star_graph(leaves):
    return fsgc.csr_from_edges(leaves + 1, [(0, i) for i in range(1, leaves + 1)])
