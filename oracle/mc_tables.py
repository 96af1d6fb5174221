"""Test infrastructure: marching-cubes tables and extraction restated for checking the library.

Cube corners, edges and faces follow RunMarchingCubesOnSdf (src/Shaders/TressFXMarchingCubes.hlsl:
147-280): corner k at offset[k], edge e between the corner pairs of its VertexLerp call.  The triangle
table is derived, not copied: on every face, walking its corners counter-clockwise seen from outside,
each crossing where the walk goes from outside to inside is joined to the next crossing where it goes
from inside to outside (on a face with four crossings this keeps the two inside corners apart); the
joined segments chain into closed loops through the shared edges, and each loop is fanned into
triangles from its first crossing."""
from __future__ import annotations

import numpy as np

CORNERS = [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1), (0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)]
EDGES = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]
# faces as corner cycles, counter-clockwise seen from outside the cube
FACES = [(0, 1, 2, 3), (4, 7, 6, 5), (0, 4, 5, 1), (3, 2, 6, 7), (0, 3, 7, 4), (1, 5, 6, 2)]


def _edge(a: int, b: int) -> int:
    for e, (p, q) in enumerate(EDGES):
        if {p, q} == {a, b}:
            return e
    raise ValueError((a, b))


def tables() -> tuple[np.ndarray, np.ndarray]:
    edge = np.zeros(256, np.int32)
    tri = -np.ones((256, 16), np.int32)
    for cfg in range(256):
        inside = [(cfg >> k) & 1 == 1 for k in range(8)]
        m = 0
        for e, (a, b) in enumerate(EDGES):
            if inside[a] != inside[b]:
                m |= 1 << e
        edge[cfg] = m
        nxt = {}
        for f in FACES:
            cross = []   # (edge, kind) in walk order; kind +1: outside -> inside, -1: inside -> outside
            for k in range(4):
                a, b = f[k], f[(k + 1) % 4]
                if inside[a] != inside[b]:
                    cross.append((_edge(a, b), 1 if inside[b] else -1))
            for i, (e, kind) in enumerate(cross):
                if kind == 1:
                    j = (i + 1) % len(cross)
                    while cross[j][1] != -1:
                        j = (j + 1) % len(cross)
                    nxt[e] = cross[j][0]
        seen, out = set(), []
        for e0 in sorted(nxt):
            if e0 in seen:
                continue
            loop, e = [], e0
            while e not in seen:
                seen.add(e)
                loop.append(e)
                e = nxt[e]
            for i in range(1, len(loop) - 1):
                out += [loop[0], loop[i], loop[i + 1]]
        tri[cfg, :len(out)] = out
    return edge, tri.reshape(-1)


def vertex_lerp(iso: np.float32, s1: np.float32, s2: np.float32, p1, p2):
    interp = np.float32((iso - s1) / (s2 - s1))
    return tuple(np.float32(a + np.float32((b - a) * interp)) for a, b in zip(p1, p2))
