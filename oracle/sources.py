"""FP64 restatement of the ray sources (oracle; tests only).

Follows utils.py:47-80 (multi_cumsum_inplace, including where its partition
counter resets), utils.py:117-175 (concentric_rings) and source.py:117-188
(PointSource / ParallelBeam generate_array, deterministic mode).
"""
from __future__ import annotations

import numpy as np


def multi_cumsum_inplace(values, partitions, start):
    part_idx = 0
    current_part_len = partitions[part_idx]
    part_count = 0
    values[0] = start
    for v_idx in range(1, values.size):
        if current_part_len == part_count:
            part_count = 0
            part_idx += 1
            current_part_len = partitions[part_idx]
            values[v_idx] = start
        else:
            values[v_idx] += values[v_idx - 1]
            part_count += 1


def concentric_rings(num_points_approx: int, radius: float) -> np.ndarray:
    num_rings = max(1, int(np.floor((-1 + np.sqrt(1 + 4 * num_points_approx / np.pi)) / 2)))
    num_points_kth_ring = np.round(2 * np.pi * np.arange(1, num_rings + 1)).astype(int)
    num_rings = num_points_kth_ring.size
    points_per_unit = num_points_approx / num_points_kth_ring.sum()
    points_per_ring = np.round(num_points_kth_ring * points_per_unit).astype(int)
    radii = np.linspace(0, radius, num_rings + 1, endpoint=True)[1:]
    with np.errstate(divide="ignore"):
        div_angle = 2 * np.pi / points_per_ring
    params = np.stack((radii, div_angle), axis=0)
    all_params = np.repeat(params, points_per_ring.tolist(), axis=-1)
    multi_cumsum_inplace(all_params[1, :], points_per_ring, 0.0)
    all_radii = all_params[0, :]
    all_angles = all_params[1, :]
    return np.stack((all_radii * np.sin(all_angles), all_radii * np.cos(all_angles)), axis=-1)


def point_source_array(num, semi_conv, offset_xy=(0.0, 0.0)):
    dy, dx = concentric_rings(num, semi_conv).T
    r = np.zeros((dx.size, 5), dtype=np.float64)
    r[:, 0] += offset_xy[0]
    r[:, 1] += offset_xy[1]
    r[:, 2] = dx
    r[:, 3] = dy
    r[:, 4] = 1.0
    return r


def parallel_beam_array(num, radius, offset_xy=(0.0, 0.0)):
    y, x = concentric_rings(num, radius).T
    r = np.zeros((x.size, 5), dtype=np.float64)
    r[:, 0] = x + offset_xy[0]
    r[:, 1] = y + offset_xy[1]
    r[:, 4] = 1.0
    return r
