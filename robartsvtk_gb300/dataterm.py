"""The data-term producers that precede a solve (libhmf_gb300.so):

* `data_term` / `ImageDataTerm` -- vtkImageDataTerm
  (Common/vtkRobartsCommon/vtkImageDataTerm.h:28-134, .cxx:28-470): constant,
  logistic, Gaussian or spike costs of one or two images, as a probability or
  an entropy, optionally normalised by the first image's range.
* `log_likelihood` / `ImageLogLikelihood` -- vtkImageLogLikelihood
  (vtkImageLogLikelihood.h, .cxx:40-250): the negative log frequency of each
  voxel's value in a histogram over seed voxels that enough label maps mark.

Images are float32 numpy arrays (host) or CUDA torch tensors (device), label
maps int32.  The facades keep the VTK method names and defaults, including
vtkImageDataTerm's SetOperationToGaussian selecting the spike code and
SetOperationToSpike the Gaussian one (vtkImageDataTerm.h:51-63).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import HMF_DEVICE, HMF_HOST, check

__all__ = ["CONSTANT", "LOGISTIC", "GAUSSIAN", "SPIKE", "data_term", "log_likelihood", "ImageDataTerm",
           "ImageLogLikelihood"]

CONSTANT, LOGISTIC, GAUSSIAN, SPIKE = 0, 1, 2, 3


def _ptr(arr, dtype):
    """(pointer, where, n, keep) of a contiguous array of `dtype`."""
    if isinstance(arr, np.ndarray):
        if arr.dtype != dtype or not arr.flags["C_CONTIGUOUS"]:
            raise TypeError("expected a C-contiguous %s array" % np.dtype(dtype).name)
        return arr.ctypes.data, HMF_HOST, arr.size, arr
    import torch

    tdt = {np.float32: torch.float32, np.int32: torch.int32}[dtype]
    if arr.dtype != tdt or not arr.is_contiguous():
        raise TypeError("expected a contiguous %s tensor" % np.dtype(dtype).name)
    return arr.data_ptr(), HMF_DEVICE if arr.is_cuda else HMF_HOST, arr.numel(), arr


def _stream(stream):
    if stream is None:
        return None
    return stream if isinstance(stream, int) else int(stream.cuda_stream)


def _new_like(arr, count=None):
    if isinstance(arr, np.ndarray):
        return np.empty(arr.shape if count is None else (count,), np.float32)
    import torch

    return torch.empty(arr.shape if count is None else (count,), dtype=torch.float32, device=arr.device)


def data_term(op, in1, in2=None, k1=1.0, c1=0.0, k2=1.0, c2=0.0, entropy=False, normalize=False, out=None,
              stream=None):
    """Per-voxel cost of `in1` (and `in2`): op = CONSTANT, LOGISTIC, GAUSSIAN or
    SPIKE (the reference's numeric codes).  Returns `out` (a new array of
    in1's shape and kind when None)."""
    lib = _capi.load()
    p1, w1, n, k_in1 = _ptr(in1, np.float32)
    p2 = None
    if in2 is not None:
        p2, w2, n2, _ = _ptr(in2, np.float32)
        if n2 != n or w2 != w1:
            raise ValueError("both images must have the same size and live on the same side")
    if out is None:
        out = _new_like(in1)
    po, wo, no, _ = _ptr(out, np.float32)
    if no != n or wo != w1:
        raise ValueError("the output must match the first image")
    check(lib.hmf_data_term(int(op), int(bool(entropy)), int(bool(normalize)), float(k1), float(c1), float(k2),
                            float(c2), p1, p2, n, po, w1, _stream(stream)))
    return out


def log_likelihood(image, label_maps, label_id=1, resolution=1.0, required_agreement=0.8, normalize=False,
                   components=1, out=None, stream=None):
    """Negative log-likelihood cost of `image` (float32, `components` = 1 or 2
    interleaved) from the seeds that at least `required_agreement` of the int32
    `label_maps` (None entries skipped) mark with `label_id`."""
    lib = _capi.load()
    pi, wi, n_el, _ = _ptr(image, np.float32)
    if n_el % components:
        raise ValueError("image size is not a multiple of the component count")
    n = n_el // components
    keep = []
    ptrs = (ctypes.c_void_p * max(1, len(label_maps)))()
    for k, m in enumerate(label_maps):
        if m is None:
            continue
        pm, wm, nm, km = _ptr(m, np.int32)
        if nm != n or wm != wi:
            raise ValueError("label maps must match the image's voxels and side")
        keep.append(km)
        ptrs[k] = pm
    if out is None:
        out = _new_like(image, n if components != 1 else None)
    po, wo, no, _ = _ptr(out, np.float32)
    if no != n or wo != wi:
        raise ValueError("the output must have one value per voxel on the image's side")
    check(lib.hmf_log_likelihood(pi, int(components), ptrs, len(label_maps), n, int(label_id),
                                 float(resolution), float(required_agreement), int(bool(normalize)), po, wi,
                                 _stream(stream)))
    return out


class ImageDataTerm:
    """vtkImageDataTerm's interface; inputs are arrays, GetOutput an array."""

    def __init__(self):
        self.Operation = CONSTANT
        self.ConstantK1 = 1.0
        self.ConstantK2 = 1.0
        self.ConstantC1 = 0.0
        self.ConstantC2 = 0.0
        self.Entropy = False
        self.Normalize = True
        self._in = [None, None]
        self._out = None

    def SetOperation(self, op):
        self.Operation = int(op)

    def GetOperation(self):
        return self.Operation

    def SetOperationToConstant(self):
        self.Operation = CONSTANT

    def SetOperationToLogistic(self):
        self.Operation = LOGISTIC

    def SetOperationToGaussian(self):  # as the reference: the spike code (vtkImageDataTerm.h:51-55)
        self.Operation = SPIKE

    def SetOperationToSpike(self):  # as the reference: the Gaussian code (vtkImageDataTerm.h:59-63)
        self.Operation = GAUSSIAN

    def SetConstantK1(self, v):
        self.ConstantK1 = float(v)

    def GetConstantK1(self):
        return self.ConstantK1

    def SetConstantK2(self, v):
        self.ConstantK2 = float(v)

    def GetConstantK2(self):
        return self.ConstantK2

    def SetConstantC1(self, v):
        self.ConstantC1 = float(v)

    def GetConstantC1(self):
        return self.ConstantC1

    def SetConstantC2(self, v):
        self.ConstantC2 = float(v)

    def GetConstantC2(self):
        return self.ConstantC2

    def SetNormalize(self, v):
        self.Normalize = bool(v)

    def GetNormalize(self):
        return self.Normalize

    def SetNormalizeOn(self):
        self.Normalize = True

    def SetNormalizeOff(self):
        self.Normalize = False

    def SetInput1Data(self, image):
        self._in[0] = image

    def SetInput2Data(self, image):
        self._in[1] = image

    def SetOutputToEntropy(self):
        self.Entropy = True

    def SetOutputToProbability(self):
        self.Entropy = False

    def GetEntropyUsed(self):
        return self.Entropy

    def GetProbabilityUsed(self):
        return not self.Entropy

    def Update(self, stream=None):
        if self._in[0] is None:
            raise ValueError("input 1 is required")
        self._out = data_term(self.Operation, self._in[0], self._in[1], self.ConstantK1, self.ConstantC1,
                              self.ConstantK2, self.ConstantC2, self.Entropy, self.Normalize and self._in[1] is None,
                              stream=stream)
        return 1

    def GetOutput(self):
        return self._out


class ImageLogLikelihood:
    """vtkImageLogLikelihood's interface; inputs are arrays, GetOutput an array."""

    def __init__(self):
        self.NormalizeDataTerm = 0
        self.LabelID = 1
        self.HistogramResolution = 1.0
        self.RequiredAgreement = 0.8
        self.Components = 1
        self._image = None
        self._maps: dict[int, object] = {}
        self._out = None

    def SetInputDataImage(self, image, components=1):
        self._image = image
        self.Components = int(components)

    def SetInputLabelMapData(self, label_map, number):
        self._maps[int(number)] = label_map

    def SetNormalizeDataTermOn(self):
        self.NormalizeDataTerm = 1

    def SetNormalizeDataTermOff(self):
        self.NormalizeDataTerm = 0

    def GetNormalizeDataTerm(self):
        return self.NormalizeDataTerm

    def SetLabelID(self, v):
        self.LabelID = max(0, int(v))

    def GetLabelID(self):
        return self.LabelID

    def SetHistogramResolution(self, v):
        self.HistogramResolution = max(float(np.finfo(np.float32).tiny), float(v))

    def GetHistogramResolution(self):
        return self.HistogramResolution

    def SetRequiredAgreement(self, v):
        self.RequiredAgreement = min(1.0, max(0.0, float(v)))

    def GetRequiredAgreement(self):
        return self.RequiredAgreement

    def Update(self, stream=None):
        if self._image is None:
            raise ValueError("an input image is required")
        n = 1 + max(self._maps) if self._maps else 0
        maps = [self._maps.get(k) for k in range(n)]
        self._out = log_likelihood(self._image, maps, self.LabelID, self.HistogramResolution, self.RequiredAgreement,
                                   self.NormalizeDataTerm, self.Components, stream=stream)
        return 1

    def GetOutput(self):
        return self._out
