"""Host side of the wave fit: the loss window's geometry (no GPU)."""
from __future__ import annotations

import numpy as np


def test_window_r2_follows_the_grid_bilerp():
    from wave_tool_gb300 import fit, workloads
    from wave_tool_gb300.abi import PATCH_DTYPE
    # two patches, the second a sheared quad written after the first
    p = np.array([workloads.square_patch(0.0, 0.0, 50.0, 5, 0, 1, 0.0, 0),
                  workloads.square_patch(0.0, 0.0, 1.0, 3, 0, 1, 0.0, 25)], dtype=PATCH_DTYPE)
    p[1]["tr"] = (3.0, -1.0)
    r2 = fit.window_r2(p, 25 + 9 + 2)
    a = r2[:25].reshape(5, 5)
    assert a[2, 2] == 0.0
    assert np.allclose(a[0, 0], 2 * 50.0 ** 2) and np.allclose(a[4, 4], 2 * 50.0 ** 2)
    assert np.allclose(a[0, 2], 50.0 ** 2) and np.allclose(a[2, 0], 50.0 ** 2)
    # patch 2: vertex (row, col) at bilerp(u = col / 2, v = row / 2), centre = mean of the corners
    bl, br, tl, tr = (np.array(p[1][k], np.float64) for k in ("bl", "br", "tl", "tr"))
    c = (bl + br + tl + tr) / 4
    for row in range(3):
        for col in range(3):
            u, v = col / 2, row / 2
            q = (1 - v) * ((1 - u) * bl + u * br) + v * ((1 - u) * tl + u * tr)
            assert np.isclose(r2[25 + 3 * row + col], ((q - c) ** 2).sum(), rtol=1e-6)
    assert np.all(r2[34:] == 0.0)  # written by no patch
