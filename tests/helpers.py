"""Comparison helpers shared by the tests."""

import numpy as np
import torch


def to_np(a):
    if torch.is_tensor(a):
        return a.detach().cpu().numpy().astype(np.float64)
    return np.asarray(a, dtype=np.float64)


def rel_l2(a, b):
    a, b = to_np(a), to_np(b)
    nb = np.linalg.norm(b.ravel())
    diff = np.linalg.norm((a - b).ravel())
    if nb == 0.0:
        return diff
    return diff / nb
