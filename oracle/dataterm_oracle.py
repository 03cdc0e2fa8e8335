"""Data-term producers restated in numpy -- TEST INFRASTRUCTURE ONLY (the oracle).

Only tests/ import this module, as the checker of hmf_data_term and
hmf_log_likelihood.  The reference filters need VTK (absent) for their
vtkImageData plumbing, so their loops are restated here, expression by
expression, in the reference's precision: double arithmetic for
vtkImageDataTerm, float histograms for vtkImageLogLikelihood.  Parity is
therefore pinned by this restatement only (no reference outputs exist).
"""
from __future__ import annotations

import numpy as np

CONSTANT, LOGISTIC, GAUSSIAN, SPIKE = 0, 1, 2, 3
F32 = np.float32


def data_term(op, in1, in2=None, k1=1.0, c1=0.0, k2=1.0, c2=0.0, entropy=False, normalize=False):
    """vtkImageDataTermExecute1 (vtkImageDataTerm.cxx:62-249) or, with in2,
    vtkImageDataTermExecute2 (:255-390); float32 images, float32 result."""
    with np.errstate(divide="ignore"):  # -log(0) of an unused default constant, as the reference
        return _data_term(op, in1, in2, k1, c1, k2, c2, entropy, normalize)


def _data_term(op, in1, in2, k1, c1, k2, c2, entropy, normalize):
    x1 = np.asarray(in1, np.float32).astype(np.float64)
    if in2 is None:
        lg = op in (CONSTANT, SPIKE) and entropy
        cc1 = -np.log(c1) if lg else c1
        cc2 = -np.log(c2) if lg else c1  # :106 -- the second constant is C1 unless it is a logarithm
        if op == CONSTANT:
            v = np.full(x1.shape, cc1)
        elif op == LOGISTIC:
            a = 1.0 + np.exp(-(k1 * (x1 - cc1)))
            v = np.log(a) if entropy else 1.0 / a
        elif op == GAUSSIAN:
            q = (x1 - cc1) / k1
            v = 0.5 * q * q if entropy else np.exp(-0.5 * q * q)
        else:
            v = np.where(x1 == k1, cc1, cc2)
        out = v.astype(np.float32)
        if not normalize:
            return out
        R0, R1 = float(np.nanmin(x1)), float(np.nanmax(x1))
        off, mul = 0.0, 1.0 / cc1
        if op == GAUSSIAN and entropy:
            vmax = 0.5 * ((R1 - cc1) / k1) * ((R1 - cc1) / k1)
            vmin = 0.5 * ((R0 - cc1) / k1) * ((R0 - cc1) / k1)
            mx = vmax if vmax >= vmin else vmin
            mn = vmax if vmax < vmin else vmin
            if R0 < cc1 < R1:
                mn = 0.0
            off, mul = -mn, 1.0 / (mx - mn)
        elif op == GAUSSIAN:
            vmax = np.exp(-0.5 * ((R1 - cc1) / k1) * ((R1 - cc1) / k1))
            vmin = np.exp(-0.5 * ((R0 - cc1) / k1) * ((R0 - cc1) / k1))
            mn = np.exp(-(vmax if vmax >= vmin else vmin))
            mx = np.exp(-(vmax if vmax < vmin else vmin))
            if R0 < cc1 < R1:
                mx = 1.0
            off, mul = -mn, 1.0 / (mx - mn)
        elif op == LOGISTIC and entropy:
            vmax = np.log(1.0 + np.exp(-(k1 * (R1 - cc1))))
            vmin = np.log(1.0 + np.exp(-(k1 * (R0 - cc1))))
            mx, mn = max(vmax, vmin), min(vmax, vmin)
            off, mul = -mn, 1.0 / (mx - mn)
        elif op == LOGISTIC:
            vmax = 1.0 / (1.0 + np.exp(-(k1 * (R1 - cc1))))
            vmin = 1.0 / (1.0 + np.exp(-(k1 * (R0 - cc1))))
            mx, mn = max(vmax, vmin), min(vmax, vmin)
            off, mul = -mn, 1.0 / (mx - mn)
        return ((out.astype(np.float64) + off) * mul).astype(np.float32)
    x2 = np.asarray(in2, np.float32).astype(np.float64)
    lg = op == CONSTANT and entropy
    cc1 = -np.log(c1) if lg else c1
    cc2 = -np.log(c2) if lg else c2
    if op == CONSTANT:
        v = np.full(x1.shape, cc1)
    elif op == LOGISTIC:
        a = 1.0 + np.exp(-(k1 * (x1 - cc1)))
        b = 1.0 + np.exp(-(k2 * (x2 - cc2)))
        v = np.log(a * b) if entropy else 1.0 / (a * b)
    elif op == GAUSSIAN:
        q1 = (x1 - cc1) / k1
        q2 = (x2 - cc2) / k2
        v = 0.5 * q1 * q1 + 0.5 * q2 * q2 if entropy else np.exp(-0.5 * q1 * q1 - 0.5 * (q2 * q2))
    else:
        raise ValueError("the reference's two-image form has no spike operation")
    return v.astype(np.float32)


def log_likelihood(image, label_maps, label_id=1, resolution=1.0, required_agreement=0.8, normalize=False,
                   components=1):
    """vtkImageLogLikelihoodExecute (vtkImageLogLikelihood.cxx:140-250) with the
    intended one-component histogram size.  Returns float32 costs per voxel;
    raises ValueError where the reference would write past its histogram."""
    img = np.asarray(image, np.float32).reshape(-1, components)
    n = img.shape[0]
    maps = [np.asarray(m).reshape(-1) for m in label_maps if m is not None]
    agree = np.zeros(n, np.int64)
    for m in maps:
        agree += (m.astype(np.int64) == int(label_id))
    sample = agree.astype(np.float64) >= float(required_agreement) * float(len(maps))
    n_sample = int(sample.sum())
    if n_sample == 0:
        return np.ones(n, np.float32)
    res = F32(resolution)
    mn = [F32(np.finfo(np.float32).max)] * 2
    mx = [F32(np.finfo(np.float32).tiny)] * 2
    for k in range(components):
        vals = img[sample, k]
        lo, hi = F32(vals.min()), F32(vals.max())
        mn[k] = mn[k] if mn[k] < lo else lo
        mx[k] = mx[k] if mx[k] > hi else hi
    sz = [1, 1]
    for k in range(components):
        sz[k] = int(np.trunc(F32(mx[k] - F32(mn[k] / res)))) + 1
        if int(np.trunc(F32(F32(mx[k] - mn[k]) / res))) >= sz[k]:
            raise ValueError("seeds span more bins than the reference's histogram holds")

    def bins(k, x):
        return np.trunc(((x - mn[k]).astype(np.float32) / res).astype(np.float32)).astype(np.int64)

    b = bins(0, img[:, 0])
    idx = b * sz[1]
    if components == 2:
        b1 = bins(1, img[:, 1])
        idx = idx + b1
    counts = np.bincount(idx[sample], minlength=sz[0] * sz[1]).astype(np.int64)
    cnt = np.minimum(counts, 1 << 24).astype(np.float32)
    freq = ((cnt / F32(n_sample)).astype(np.float64) + 1.0e-10).astype(np.float32)
    floor = -np.log(1.0e-10)
    outside = (img[:, 0] < mn[0]) | (b >= sz[0])
    if components == 2:
        outside |= (img[:, 1] < mn[1]) | (b1 >= sz[1])
    safe = np.where(outside, 0, idx)
    out = np.where(outside, F32(floor), (-np.log(freq[safe].astype(np.float64))).astype(np.float32))
    out = out.astype(np.float32)
    if normalize:
        out = (out.astype(np.float64) / floor).astype(np.float32)
    return out
