"""CPU restatement of goal's isotropic target size field -- TEST INFRASTRUCTURE ONLY.

get_iso_target_size (src/goal_size_field.cpp:139-151) with d = 3, p = 1:
  G       = sum_e |theta_e|^(2d/(2p+d))                         (:39-52)
  factor  = (G / target)^(1/d)                                  (:54-59)
  h_e     = sqrt(sum of squared edge lengths / 6)               (:61-68)
  h_new_e = factor |theta_e|^(-2/(2p+d)) h_e, clamped to [alpha h_e, beta h_e],
            alpha = 0.25, beta = 2                              (:70-81, :29-30)
  size_v  = mean of h_new over the elements adjacent to v       (:96-106)
"""
from __future__ import annotations

import numpy as np

EDGES = ((0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3))


def element_sizes(coords, tets):
    h = np.zeros(len(tets))
    for a, b in EDGES:
        d = coords[tets[:, a]] - coords[tets[:, b]]
        h += (d * d).sum(axis=1)
    return np.sqrt(h / 6.0)


def iso_target_size(coords, tets, err, target, d=3, p=1, alpha=0.25, beta=2.0):
    theta = np.abs(np.asarray(err, dtype=np.float64))
    G = np.sum(theta ** ((2.0 * d) / (2.0 * p + d)))
    factor = (G / target) ** (1.0 / d)
    h = element_sizes(coords, tets)
    with np.errstate(divide="ignore"):
        r = theta ** (-2.0 / (2.0 * p + d))
    hn = np.clip(factor * r * h, alpha * h, beta * h)
    N = len(coords)
    s = np.zeros(N)
    cnt = np.zeros(N)
    for a in range(4):
        np.add.at(s, tets[:, a], hn)
        np.add.at(cnt, tets[:, a], 1.0)
    return np.where(cnt > 0, s / np.maximum(cnt, 1.0), 0.0)
