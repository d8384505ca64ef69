"""Strand file ingest and arclength resampling, with the reference package's signatures
(``pystrns2cards/__init__.py:42-107``): ``load_strands``, ``resample_strands_by_arclength``,
``load_strands_arc_length``.  File parsing is host C++ in libs2c; resampling runs on the
host for numpy arrays (as the reference) and on the device for CUDA tensors, with results
identical between the two."""
from __future__ import annotations

import numpy as np
import torch

from . import _core


def load_strands(filepath: str, return_raw: bool = False):
    """(N,) object array of (M_i, 3) float32 strands; with ``return_raw`` also the flat
    (num_samples, points) arrays."""
    num_samples, points = _core.load_strands(filepath)
    num_samples = np.asarray(num_samples).ravel()
    strands = np.empty(len(num_samples), dtype=object)
    offs = np.concatenate([[0], np.cumsum(num_samples)])
    for i in range(len(num_samples)):
        strands[i] = points[offs[i]:offs[i + 1]]
    if offs[-1] != len(points):
        raise RuntimeError("load_strands: Offset mismatch after slicing points.")
    return (strands, num_samples, points) if return_raw else strands


def resample_strands_by_arclength(num_samples, points, target_num_samples: int = 100):
    """(N, target, 3) float32: each strand resampled to points evenly spaced in arclength.
    CUDA tensors are resampled on the device (a CUDA tensor is returned), numpy on the host."""
    if isinstance(points, torch.Tensor) and points.is_cuda:
        ns = torch.as_tensor(num_samples, dtype=torch.int32, device=points.device).reshape(-1).contiguous()
        return _core.resample_strands_by_arclength_device(ns, points.float().reshape(-1, 3).contiguous(),
                                                          target_num_samples)
    return _core.resample_strands_by_arclength(np.asarray(num_samples).ravel(), np.asarray(points),
                                               target_num_samples)


def load_strands_arc_length(filepath: str, target_num_samples: int = 100) -> np.ndarray:
    """Load and resample to ``target_num_samples`` points per strand."""
    num_samples, points = _core.load_strands(filepath)
    return resample_strands_by_arclength(num_samples, points, target_num_samples)
