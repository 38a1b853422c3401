"""FP64 restatement of the transfer-matrix helpers (oracle; tests only).

Follows transfer.py:6-53 (transfer_rays), 56-112 (transfer_rays_pt_src),
115-137 (accumulate_matrices) and 140-183 (accumulate_matrices_cumulative),
including the cumulative loop's actual order: it starts from the LAST
matrix and multiplies the earlier ones on the left.
"""
from __future__ import annotations

import numpy as np


def accumulate_matrices(matrices):
    total = matrices[-1]
    for tm in reversed(matrices[:-1]):
        total = total @ tm
    return total


def accumulate_matrices_cumulative(matrices):
    out = []
    total = matrices[-1]
    out.append(total)
    for tm in reversed(matrices[:-1]):
        total = tm @ total
        out.append(total)
    return np.stack(out, axis=0)


def transfer_rays(ray_coords, transfer_matrices):
    cum = accumulate_matrices_cumulative(np.asarray(transfer_matrices, np.float64))
    return np.einsum("mij,nj->nmi", cum, np.asarray(ray_coords, np.float64))


def transfer_rays_pt_src(input_pos_xy, input_slopes_xy, transfer_matrix):
    x0, y0 = input_pos_xy
    sx, sy = (np.asarray(v, np.float64) for v in input_slopes_xy)
    v = np.vstack([np.full(sx.shape[0], x0), np.full(sy.shape[0], y0), sx, sy, np.ones_like(sx)])
    end = np.asarray(transfer_matrix, np.float64) @ v
    return end[:4]
