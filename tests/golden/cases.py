"""Small seeded HMF problems shared by the golden-vector generator and the
tests.  Inputs are regenerated from the seed (numpy's PCG64 stream is the same
on every platform); only outputs are stored in the .npz fixtures."""
from robartsvtk_gb300.synthetic import random_tree_problem

# name: (seed, (VX, VY, VZ), parent, iterations, vertices with a smoothness image)
CASES = {
    "tree2_7x5x4": (11, (7, 5, 4), [-1, 0, 0, 1, 1, 2, 2], 50, (1, 3, 6)),
    "flat3_13x6x9": (12, (13, 6, 9), [-1, 0, 0, 0], 40, ()),
    "tree3_33x9x17": (13, (33, 9, 17), [-1, 0, 0, 1, 1, 2, 3, 3, 4, 4], 30, (2, 5, 7)),
    "flat2_1x8x5": (14, (1, 8, 5), [-1, 0, 0], 25, (1,)),
    "chain_6x7x3": (15, (6, 7, 3), [-1, 0, 1, 1, 0], 35, (3,)),
}


def problem(name):
    seed, dims, parent, iters, smooth_nodes = CASES[name]
    return random_tree_problem(seed, dims, parent, iterations=iters, smooth_nodes=smooth_nodes)

# vote and energy-decomposition cases: name -> (seed, (VX, VY, VZ), vote inputs)
POST_CASES = {
    "post_9x7x5": (21, (9, 7, 5), 4),
    "post_1x13x4": (22, (1, 13, 4), 3),
    "post_31x2x3": (23, (31, 2, 3), 5),
}


def post_problem(name):
    """Vote inputs quantised to a few levels (so that ties occur), their ids,
    one labelling and one smoothness image."""
    import numpy as np

    seed, dims, n_in = POST_CASES[name]
    rng = np.random.default_rng(seed)
    shape = dims[::-1]
    inputs = [(rng.integers(0, 4, size=shape) / 4.0).astype(np.float32) for _ in range(n_in)]
    values = [int(v) for v in rng.permutation(10)[:n_in]]
    label = rng.random(shape).astype(np.float32)
    smooth = rng.random(shape).astype(np.float32)
    return {"dims": dims, "inputs": inputs, "values": values, "label": label, "smooth": smooth}

# DAG solver cases: name -> (seed, (VX, VY, VZ), n_nodes, edges, weights or None,
# iterations, vertices with a smoothness image)
DAG_CASES = {
    "dag_diamond_9x7x5": (31, (9, 7, 5), 6, [(0, 1), (0, 2), (1, 3), (2, 3), (1, 4), (2, 5)], None, 20, (1, 3)),
    "dag_weighted_11x6x7": (32, (11, 6, 7), 7, [(0, 1), (0, 2), (0, 3), (1, 4), (1, 5), (2, 5), (2, 6)],
                            [1.0, 0.5, 2.0, 1.5, 0.25, 0.75, 1.0], 15, (2, 5)),
    "dag_skip_13x5x3": (33, (13, 5, 3), 6, [(0, 1), (1, 2), (2, 3), (2, 4), (0, 4), (1, 5)], None, 25, ()),
    "dag_tree_8x8x4": (34, (8, 8, 4), 7, [(0, 1), (0, 2), (1, 3), (1, 4), (2, 5), (2, 6)], None, 12, (4,)),
}


class DagProblem:
    def __init__(self, dims, n, edges, weights, data, smooth, alpha, iterations, step=0.1, cc=0.25):
        self.dims, self.n, self.edges, self.weights = dims, n, edges, weights
        self.data, self.smooth, self.alpha = data, smooth, alpha
        self.iterations, self.step, self.cc = iterations, step, cc
        kids = {p for p, _ in edges}
        self.leaves = [v for v in range(n) if v not in kids]


def dag_problem(name):
    """Uniform data terms on the leaves, uniform smoothness images on the listed
    vertices, a seeded alpha on every non-root vertex."""
    import numpy as np

    seed, dims, n, edges, weights, iters, smooth_nodes = DAG_CASES[name]
    rng = np.random.default_rng(seed)
    shape = dims[::-1]
    parents = {c for _, c in edges}
    kids = {p for p, _ in edges}
    data = {v: rng.uniform(0, 3.0, size=shape).astype(np.float32) for v in range(n) if v not in kids}
    smooth = {v: rng.uniform(0, 1, size=shape).astype(np.float32) for v in smooth_nodes}
    alpha = {v: float(rng.uniform(0.05, 1.0)) for v in range(n) if v in parents}
    return DagProblem(dims, n, edges, weights, data, smooth, alpha, iters)
