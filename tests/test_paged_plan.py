"""The out-of-core solve's block layout and its temporal blocking, on the CPU.

An hmf_create_paged context keeps the whole state in host memory and
iterates it in rounds of k iterations: each block of T z-planes is iterated
k times on its own, its faces taking the volume-face rules, and keeps only
the planes it owns, which lie at least H = 2k + 1 planes from every face
inside the volume.  hmf_paged_layout (host only) places the blocks.  Here
the oracle runs that schedule block by block and must reproduce the
monolithic solve bit for bit (flows, divergence, labels and sinks of every
vertex); with one halo plane too few it must not.

The device's flow step forms the old divergence from the stored flows
instead of reading the divergence array; at a block's top plane that lacks
the z-flow of the plane above, which is why the high-z side needs the extra
plane.  The oracle reads the divergence array, so each block's divergence is
replaced by that recomputation when the block is loaded."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from robartsvtk_gb300.synthetic import random_tree_problem

PARENT = [-1, 0, 0, 1, 1, 2, 2]
KEYS = ("fx", "fy", "fz", "div", "u", "sink")


def layout(lib, vz, T, H):
    n = lib.hmf_paged_layout(vz, T, H, None, None, 0)
    if n < 0:
        return None
    starts = (ctypes.c_int * n)()
    owned = (ctypes.c_int * n)()
    assert lib.hmf_paged_layout(vz, T, H, starts, owned, n) == n
    return list(starts), list(owned)


@pytest.mark.parametrize("vz", [1, 7, 16, 40, 97, 256, 384])
@pytest.mark.parametrize("T,H", [(8, 2), (16, 4), (24, 6), (33, 8), (64, 16), (96, 16), (500, 4), (12, 0)])
def test_layout_covers_the_volume_with_exact_owned_planes(hmf_lib, vz, T, H):
    got = layout(hmf_lib, vz, T, H)
    assert got is not None
    starts, owned = got
    nb = len(starts)
    Tb = min(T, vz)
    assert starts[0] == 0 and owned[0] == 0 and starts[-1] + Tb == vz
    bounds = owned + [vz]
    for j in range(nb):
        b, a0, a1 = starts[j], bounds[j], bounds[j + 1]
        assert a0 < a1
        # owned planes are exact: at least H planes from an inner face
        lo = b if j == 0 else b + H
        hi = b + Tb if j == nb - 1 else b + Tb - H
        assert lo <= a0 and a1 <= hi, (j, b, a0, a1)
        # a block's owned planes are read by its neighbours only, so the
        # store of block j can wait for the load of block j+1 alone
        if j + 2 < nb:
            assert starts[j + 2] >= a1
    if nb > 1:
        assert nb == 1 + -(-(vz - Tb) // (Tb - 2 * H))


def test_block_count_never_grows_with_thicker_blocks(hmf_lib):
    """The out-of-core plan shrinks a budget-derived block to the thinnest
    one with the same block count, found by bisection: that needs the count
    to be non-increasing in the block thickness (from 4 x halo up)."""
    for vz in (45, 96, 256, 384, 1000):
        for H in (3, 5, 19, 23, 25):
            counts = [hmf_lib.hmf_paged_layout(vz, T, H, None, None, 0) for T in range(4 * H, vz + 2)]
            assert all(c > 0 for c in counts)
            assert all(a >= b for a, b in zip(counts, counts[1:])), (vz, H)


def test_layout_rejects_blocks_thinner_than_four_halos(hmf_lib):
    assert hmf_lib.hmf_paged_layout(100, 15, 4, None, None, 0) == -1
    assert hmf_lib.hmf_paged_layout(100, 16, 4, None, None, 0) > 0
    assert hmf_lib.hmf_paged_layout(10, 15, 4, None, None, 0) == 1  # one block covers the volume
    assert hmf_lib.hmf_paged_layout(0, 8, 0, None, None, 0) == -1


def face_divergence(st):
    """The divergence the flow step forms from a block's stored flows, in its
    operation order: ((px + py) + pz) - px(x+1) - py(y+1) - pz(z+1), each
    neighbour term dropped at the block's last column, row and plane."""
    fx, fy, fz = st["fx"], st["fy"], st["fz"]
    d = (fx + fy) + fz
    d[..., :-1] = d[..., :-1] - fx[..., 1:]
    d[..., :-1, :] = d[..., :-1, :] - fy[..., 1:, :]
    d[:, :-1] = d[:, :-1] - fz[:, 1:]
    return d


def blocked_solve(w, starts, owned, k):
    """The out-of-core schedule with the oracle as the block solver."""
    vx, vy, vz = w.dims
    n = len(w.parent)
    T = vz - starts[-1]  # the last block ends at the volume's last plane
    host = O.new_state(w.dims, n)
    rounds = []
    left = w.iterations
    while left > 0:
        rounds.append(min(k, left))
        left -= rounds[-1]
    bounds = owned + [vz]
    for r, kr in enumerate(rounds):
        new = {key: host[key].copy() for key in KEYS}
        for j, b in enumerate(starts):
            sl = slice(b, b + T)
            dims = (vx, vy, T)
            data = {v: np.ascontiguousarray(d[sl]) for v, d in w.data.items()}
            smooth = {v: np.ascontiguousarray(S[sl]) for v, S in w.smooth.items()}
            st = O.new_state(dims, n)
            if r > 0:
                for key in KEYS:
                    st[key][...] = host[key][:, sl]
                st["div"][...] = face_divergence(st)
            O.iterate(dims, w.parent, data, st, smooth, w.alpha, iterations=kr, step=w.step, cc=w.cc,
                      init=(r == 0), threads=1)
            a0, a1 = bounds[j], bounds[j + 1]
            for key in KEYS:
                new[key][:, a0:a1] = st[key][:, a0 - b:a1 - b]
        host = new
    return host


@pytest.mark.parametrize("dims,T,k,iterations", [
    ((13, 11, 40), 20, 2, 11),   # 3 blocks, a short last round
    ((13, 11, 50), 20, 2, 11),   # owned planes exactly 2k+1 from the top faces
    ((9, 12, 37), 28, 3, 9),     # 2 blocks, rounds of 3
    ((10, 7, 29), 12, 1, 5),     # thinnest blocks for k = 1
    ((11, 9, 20), 32, 4, 10),    # one block covers the volume
])
def test_blocked_rounds_equal_the_monolithic_solve(hmf_lib, dims, T, k, iterations):
    w = random_tree_problem(7, dims, PARENT, iterations=iterations, smooth_nodes=(1, 4))
    mono = O.new_state(w.dims, len(PARENT))
    O.iterate(w.dims, PARENT, w.data, mono, w.smooth, w.alpha, iterations=w.iterations, step=w.step, cc=w.cc,
              init=True, threads=1)
    H = 0 if T >= dims[2] else 2 * k + 1
    starts, owned = layout(hmf_lib, dims[2], T, H)
    got = blocked_solve(w, starts, owned, k if T < dims[2] else iterations)
    for key in KEYS:
        rows = [v for v in range(len(PARENT)) if key == "sink" or PARENT[v] >= 0]
        for v in rows:
            assert np.array_equal(got[key][v], mono[key][v]), (key, v)


def test_one_halo_plane_too_few_changes_the_result(hmf_lib):
    """2k planes of halo leave the top faces' extra reach uncovered where a
    block owns planes exactly 2k from its top face (T = 16, vz = 45)."""
    w = random_tree_problem(8, (37, 19, 45), PARENT, iterations=8, smooth_nodes=(1,))
    mono = O.new_state(w.dims, len(PARENT))
    O.iterate(w.dims, PARENT, w.data, mono, w.smooth, w.alpha, iterations=w.iterations, step=w.step, cc=w.cc,
              init=True, threads=1)
    k = 2
    starts, owned = layout(hmf_lib, 45, 16, 2 * k)
    got = blocked_solve(w, starts, owned, k)
    assert any(not np.array_equal(got[key], mono[key]) for key in KEYS)
