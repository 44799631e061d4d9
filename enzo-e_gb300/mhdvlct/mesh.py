"""Leaf blocks of a periodic root grid refined by octree splitting, and the
faces of Cello's ghost refresh between them.

Cello refreshes ghost zones by letting every leaf block send to each
neighbouring leaf that its neighbour iterator yields
(Block::refresh_load_field_faces_, src/Cello/control_refresh.cpp:243-329;
ItNeighbor::valid_, src/Cello/mesh_ItNeighbor.cpp:200-265, with min face rank
0 so that edges and corners count):
  - a same-level neighbour across the face;
  - the parent of the same-level position when that position lies in a
    coarser leaf -- only for faces that point out of the sender's own parent
    along every non-zero axis, so that no coarse block is sent to twice;
  - the children of the same-level position adjacent to the face when that
    position is refined.
`Mesh.faces()` yields those (sender, receiver) pairs as the C ABI's
MhdRefreshFace records.  The mesh needs the 2:1 balance Cello keeps (a leaf's
neighbours are at most one level apart).
"""
from __future__ import annotations

import itertools

import numpy as np

from . import capi

DIRECTIONS = [f for f in itertools.product((-1, 0, 1), repeat=3)
              if f != (0, 0, 0)]


class Mesh:
    """Leaves of a periodic grid of `root_blocks` root blocks, each split into
    eight children wherever `refine(level, coords)` is true, down to
    `max_level`.  coords are (ix, iy, iz) at that level."""

    def __init__(self, root_blocks, refine=None, max_level=1):
        self.root = tuple(int(x) for x in root_blocks)
        self.max_level = int(max_level)
        leaves = []
        todo = [(0, c) for c in itertools.product(*[range(r) for r in self.root])]
        while todo:
            lvl, c = todo.pop()
            if refine is not None and lvl < self.max_level and refine(lvl, c):
                for k in itertools.product((0, 1), repeat=3):
                    todo.append((lvl + 1, tuple(2 * c[a] + k[a] for a in range(3))))
            else:
                leaves.append((lvl, c))
        # coarse first, then z, y, x
        leaves.sort(key=lambda t: (t[0], t[1][2], t[1][1], t[1][0]))
        self.leaves = leaves
        self._index = {t: i for i, t in enumerate(leaves)}
        self._refined = set()
        for lvl, c in leaves:
            for up in range(lvl):
                shift = lvl - up
                self._refined.add((up, tuple(x >> shift for x in c)))

    def extent(self, level):
        return tuple(r << level for r in self.root)

    def leaf(self, level, c):
        """Index of the leaf at (level, c), or None."""
        return self._index.get((level, tuple(c)))

    def faces(self):
        """The refresh faces of every leaf, as MhdRefreshFace tuples
        (sender, receiver, type, face, child)."""
        out = []
        for s, (lvl, c) in enumerate(self.leaves):
            ext = self.extent(lvl)
            for f in DIRECTIONS:
                p = tuple((c[a] + f[a]) % ext[a] for a in range(3))
                r = self.leaf(lvl, p)
                if r is not None:
                    out.append((s, r, capi.MHD_REFRESH_SAME, f, (0, 0, 0)))
                    continue
                if (lvl, p) in self._refined:
                    # children of p adjacent to the face
                    choices = [(0,) if f[a] == 1 else (1,) if f[a] == -1 else (0, 1)
                               for a in range(3)]
                    for k in itertools.product(*choices):
                        q = tuple(2 * p[a] + k[a] for a in range(3))
                        r = self.leaf(lvl + 1, q)
                        if r is None:
                            raise ValueError("mesh is not 2:1 balanced")
                        out.append((s, r, capi.MHD_REFRESH_FINE, f, k))
                    continue
                parent = tuple(x >> 1 for x in p)
                r = self.leaf(lvl - 1, parent) if lvl > 0 else None
                if r is None:
                    raise ValueError("mesh is not 2:1 balanced")
                own = tuple(x & 1 for x in c)
                if any((f[a] == 1 and own[a] == 0) or (f[a] == -1 and own[a] == 1)
                       for a in range(3)):
                    continue  # reached through a face that leaves the parent
                out.append((s, r, capi.MHD_REFRESH_COARSE, f, own))
        return out

    def face_array(self):
        """faces() as a ctypes array of MhdRefreshFace."""
        fs = self.faces()
        arr = (capi.MhdRefreshFace * max(1, len(fs)))()
        for i, (s, r, t, f, k) in enumerate(fs):
            arr[i].sender, arr[i].receiver, arr[i].type = s, r, t
            for a in range(3):
                arr[i].face[a] = f[a]
                arr[i].child[a] = k[a]
        return arr, len(fs)

    def face_ints(self):
        """faces() as an int32 array of 9 per face (the oracle's layout)."""
        fs = self.faces()
        return np.array([[s, r, t, *f, *k] for s, r, t, f, k in fs],
                        dtype=np.int32).reshape(-1, 9)

    def origin(self, i, n):
        """Lower corner of leaf i in cells of the finest level, for blocks of
        n active cells per axis."""
        lvl, c = self.leaves[i]
        scale = 1 << (self.max_level - lvl)
        return tuple(c[a] * n[a] * scale for a in range(3))
