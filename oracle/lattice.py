"""D2Q9 and D3Q19 velocity sets and per-face boundary tables.

The numbering, weights and face tables must be identical to the reference's, since
every array the reference produces is indexed by them:
vivsim/lbm/lattice.py:39-110 (D2Q9) and vivsim/lbm3d/lattice.py:39-126 (D3Q19).
"""

from typing import NamedTuple

import numpy as np


class Face2D(NamedTuple):
    wall: tuple
    neighbor: tuple
    in_dirs: tuple
    out_dirs: tuple
    tan_dirs: tuple
    pos_side_dirs: tuple
    neg_side_dirs: tuple
    normal_sign: int
    normal_axis: int


class Face3D(NamedTuple):
    wall: tuple
    neighbor: tuple
    in_dirs: tuple
    out_dirs: tuple
    zero_dirs: tuple
    normal_sign: int
    normal_axis: int
    tangential_axes: tuple


# ----------------------------------------------------------------------- D2Q9
# vivsim/lbm/lattice.py:39-61
Q9_W = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4, dtype=np.float32)
Q9_C = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1],
                 [1, 1], [-1, 1], [-1, -1], [1, -1]], dtype=np.int32)
Q9_OPP = (0, 3, 4, 1, 2, 7, 8, 5, 6)
Q9_RIGHT = (1, 5, 8)
Q9_LEFT = (3, 7, 6)
Q9_UP = (2, 5, 6)
Q9_DOWN = (4, 7, 8)

# vivsim/lbm/lattice.py:62-109
Q9_FACES = {
    "left": Face2D((0,), (1,), (1, 5, 8), (3, 7, 6), (2, 4), (2, 5, 6), (4, 7, 8), 1, 0),
    "right": Face2D((-1,), (-2,), (3, 7, 6), (1, 5, 8), (2, 4), (2, 5, 6), (4, 7, 8), -1, 0),
    "top": Face2D((slice(None), -1), (slice(None), -2), (4, 7, 8), (2, 5, 6), (1, 3),
                  (1, 5, 8), (3, 7, 6), -1, 1),
    "bottom": Face2D((slice(None), 0), (slice(None), 1), (2, 5, 6), (4, 7, 8), (1, 3),
                     (1, 5, 8), (3, 7, 6), 1, 1),
}

# ---------------------------------------------------------------------- D3Q19
# vivsim/lbm3d/lattice.py:39-67
Q19_W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, dtype=np.float32)
Q19_C = np.array([
    [0, 0, 0],
    [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
    [1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0],
    [1, 0, 1], [-1, 0, 1], [1, 0, -1], [-1, 0, -1],
    [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1],
], dtype=np.int32)
Q19_OPP = (0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15)
Q19_CS2 = 1.0 / 3.0

_S = slice(None)
# vivsim/lbm3d/lattice.py:68-125
Q19_FACES = {
    "left": Face3D((0, _S, _S), (1, _S, _S), (1, 7, 9, 11, 13), (2, 8, 10, 12, 14),
                   (0, 3, 4, 5, 6, 15, 16, 17, 18), 1, 0, (1, 2)),
    "right": Face3D((-1, _S, _S), (-2, _S, _S), (2, 8, 10, 12, 14), (1, 7, 9, 11, 13),
                    (0, 3, 4, 5, 6, 15, 16, 17, 18), -1, 0, (1, 2)),
    "bottom": Face3D((_S, 0, _S), (_S, 1, _S), (3, 7, 8, 15, 17), (4, 9, 10, 16, 18),
                     (0, 1, 2, 5, 6, 11, 12, 13, 14), 1, 1, (0, 2)),
    "top": Face3D((_S, -1, _S), (_S, -2, _S), (4, 9, 10, 16, 18), (3, 7, 8, 15, 17),
                  (0, 1, 2, 5, 6, 11, 12, 13, 14), -1, 1, (0, 2)),
    "back": Face3D((_S, _S, 0), (_S, _S, 1), (5, 11, 12, 15, 16), (6, 13, 14, 17, 18),
                   (0, 1, 2, 3, 4, 7, 8, 9, 10), 1, 2, (0, 1)),
    "front": Face3D((_S, _S, -1), (_S, _S, -2), (6, 13, 14, 17, 18), (5, 11, 12, 15, 16),
                    (0, 1, 2, 3, 4, 7, 8, 9, 10), -1, 2, (0, 1)),
}
