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
