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
