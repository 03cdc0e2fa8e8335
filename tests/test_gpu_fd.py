"""Gradients of the adjoint (hmf_solve_adjoint) against FP64 central finite
differences at full size.  GPU only.

Workload: 128^3, 4 ellipsoids, noise sigma 0.1, flat tree of 4 leaves, data
terms D_k = Gaussian NLL + a learnable per-voxel offset o_k (0 here, the
offset clamped so that D >= 0), one learnable alpha_k = 0.1 per leaf, 300
iterations with checkpoints every 30, loss = voxelwise cross-entropy
-(1/V) sum log(max(u_truth, eps)) of the final labels.

Finite differences: the same iteration evaluated in FP64 on the GPU
(hmf_solve_fp64 with a probe on one input), h = 1e-3, central quotient
(L(+h) - L(-h)) / 2h, at 64 seeded (leaf, voxel) offsets and at every alpha.
A probe whose two one-sided quotients disagree, (L(+h) - L(0))/h against
(L(0) - L(-h))/h, straddles a kink of the piecewise-smooth map (a capacity
clamp, a saturated label or a projection switching inside [-h, h]); such
probes are reported and left out of the bar.

Bar: on every other probe |g_adjoint - g_fd| <= RTOL |g_fd| + ATOL.  The
adjoint differentiates the FP32 forward pass, the quotients the FP64 one, so
the bar allows for the FP32 trajectory's distance from the FP64 one.
"""
import numpy as np
import pytest

from robartsvtk_gb300 import HMFSolver
from robartsvtk_gb300._capi import HMF_FP64_PROBE_ALPHA, HMF_FP64_PROBE_DATA, HMF_FP64_PROBE_NONE
from robartsvtk_gb300.synthetic import ellipsoids_flat4

pytestmark = pytest.mark.gpu
H = 1e-3
EPS = 1e-6
RTOL = 2e-2   # relative bar on non-kink probes (FP32 adjoint against FP64 differences)
KINK = 0.1    # one-sided quotients further apart than this (relative) mark a kink
N_PROBES = 64


def test_adjoint_against_fp64_central_differences():
    w = ellipsoids_flat4(seed=3, size=128, iterations=300)
    truth_leaf = np.ascontiguousarray(w.truth, dtype=np.int32)  # phantom class k is leaf index k
    V = w.nvox
    atol = 1e-3 / V  # the loss is a mean over V voxels: per-voxel gradients are O(1/V)
    rng = np.random.default_rng(2024)
    with HMFSolver(w.dims, w.parent) as s:
        for leaf, d in w.data.items():
            s.set_data(leaf, d)
        for v, a in w.alpha.items():
            s.set_smoothness_scalar(v, a)
        s.set_params(w.iterations, w.step, w.cc)
        loss32 = s.solve_adjoint(truth_leaf, checkpoint_every=30, eps=EPS)
        plan = s.adjoint_plan()
        grads = {leaf: s.data_gradient(leaf).reshape(-1) for leaf in w.leaves}
        galpha = s.alpha_gradient()

        def fp64_loss(probe=None):
            s.set_fp64_probe(HMF_FP64_PROBE_NONE)
            if probe is not None:
                s.set_fp64_probe(*probe)
            s.solve_fp64()
            return s.fp64_loss(truth_leaf, eps=EPS)

        L0 = fp64_loss()
        rows = []
        leaves = w.leaves
        picks = [(leaves[int(rng.integers(len(leaves)))], int(rng.integers(V))) for _ in range(N_PROBES)]
        for leaf, vox in picks:
            nll = float(w.data[leaf].reshape(-1)[vox])  # offset 0: D = max(NLL + o, 0)
            lp = fp64_loss((HMF_FP64_PROBE_DATA, leaf, vox, max(nll + H, 0.0)))
            lm = fp64_loss((HMF_FP64_PROBE_DATA, leaf, vox, max(nll - H, 0.0)))
            rows.append(("offset", leaf, vox, float(grads[leaf][vox]), lp, lm))
        for v in leaves:
            a = float(np.float32(w.alpha[v]))
            lp = fp64_loss((HMF_FP64_PROBE_ALPHA, v, 0, a + H))
            lm = fp64_loss((HMF_FP64_PROBE_ALPHA, v, 0, a - H))
            rows.append(("alpha", v, -1, float(galpha[v]), lp, lm))
        s.set_fp64_probe(HMF_FP64_PROBE_NONE)

    checked, kinks, worst, nonzero, bad = 0, [], 0.0, 0, []
    for kind, node, vox, g, lp, lm in rows:
        fd = (lp - lm) / (2 * H)
        fwd, bwd = (lp - L0) / H, (L0 - lm) / H
        scale = max(abs(fwd), abs(bwd), atol)
        kink = abs(fwd - bwd) > KINK * scale
        err = abs(g - fd)
        print("%-6s node %d voxel %8d  adjoint % .6e  fd % .6e  fwd % .6e  bwd % .6e  rel %.3g%s"
              % (kind, node, vox, g, fd, fwd, bwd, err / (abs(fd) + atol), "  KINK" if kink else ""))
        if kink:
            kinks.append((kind, node, vox))
            continue
        worst = max(worst, err / (abs(fd) + atol))
        nonzero += abs(fd) > atol
        checked += 1
        if err > RTOL * abs(fd) + atol:
            bad.append((kind, node, vox, g, fd))
    print("FD check, 128^3 flat4, 300 iterations, checkpoints every %d (%d recomputed segments): loss fp32 %.9f, "
          "fp64 %.9f; %d probes checked (%d with |g| above %.1e), worst relative error %.3g; %d kink hits: %s"
          % (plan["checkpoint_every"], plan["recomputed_segments"], loss32, L0, checked, nonzero, atol, worst,
             len(kinks), kinks))
    assert not bad, bad
    assert checked >= len(rows) // 2
