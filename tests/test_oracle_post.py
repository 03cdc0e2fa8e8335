"""The oracle's vote and energy decomposition against the reference kernels'
own outputs (tests/golden/ref_post_golden.npz, made by
tests/golden/make_golden.py --ref-post from CUDA_imagevote.cu and
CUDA_hierarchicalmaxflowdecomp.cu compiled unmodified): votes and per-voxel
gradient terms bit-identical.  CPU only."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_post_golden.npz")


def cases():
    g = np.load(GOLDEN)
    return g, sorted({k.split("/")[0] for k in g.files})


def test_vote_matches_reference_kernel():
    g, names = cases()
    for name in names:
        got = O.vote(list(g[name + "/vote_inputs"]), g[name + "/vote_values"], semantics=O.REF_CUDA)
        assert np.array_equal(got, g[name + "/vote"]), name


def test_gradient_terms_match_reference_kernel():
    g, names = cases()
    for name in names:
        lab = g[name + "/label"]
        dims = lab.shape[::-1]
        zero = np.zeros_like(lab)
        plain = O.energy(dims, [-1, 0, 0], {1: zero, 2: zero}, {1: lab, 2: zero}, want_terms=True)
        assert np.array_equal(plain["terms"][1], g[name + "/grad"]), name
        sm = O.energy(dims, [-1, 0, 0], {1: zero, 2: zero}, {1: lab, 2: zero}, smooth={1: g[name + "/smooth"]},
                      want_terms=True)
        assert np.array_equal(sm["terms"][1], g[name + "/grad_smooth"]), name


def test_vote_tie_rules():
    a = np.array([1.0, 2.0, 2.0, 0.0], np.float32)
    b = np.array([1.0, 2.0, 1.0, 0.0], np.float32)
    # vtkCudaImageVote: the last input of a tie wins; vtkImageVote: the first
    assert O.vote([a, b], [5, 7], semantics=O.REF_CUDA).tolist() == [7, 7, 5, 7]
    assert O.vote([a, b], [5, 7], semantics=O.REF_CPU).tolist() == [5, 5, 5, 5]


def test_branch_labelling_is_the_sum_of_its_children():
    rng = np.random.default_rng(3)
    shape = (4, 5, 6)
    dims = shape[::-1]
    lab = {2: rng.random(shape).astype(np.float32), 3: rng.random(shape).astype(np.float32),
           4: rng.random(shape).astype(np.float32)}
    dat = {k: rng.random(shape).astype(np.float32) for k in lab}
    tree = O.energy(dims, [-1, 0, 1, 1, 0], dat, lab, want_terms=True)
    # vertex 1 = {2, 3}: its term equals that of a leaf holding lab2 + lab3
    flat = O.energy(dims, [-1, 0, 0], {1: dat[2], 2: dat[4]}, {1: lab[2] + lab[3], 2: lab[4]}, want_terms=True)
    assert np.array_equal(tree["terms"][1], flat["terms"][1])
    assert tree["f"][0] == 0.0
    with pytest.raises(RuntimeError):
        O.energy(dims, [-1, 0, 0], {1: dat[2]}, {1: lab[2]})
