"""Marching-cubes mesh extraction restated on the CPU -- TEST INFRASTRUCTURE.

The reference extracts one surface mesh per structural element from the
dense-grid scalar field of its series (``gempy/modules/mesh_extranction/
marching_cubes.py:12-56``): the isovalue is the element's
``scalar_field_at_interface``, the mask is the series' squeezed mask
(``combined_scalar_field.squeezed_mask_array``; all points for a FAULT
series), and the call is ``skimage.measure.marching_cubes(..., mask=mask,
method="lewiner")`` (``marching_cubes.py:86-93``), with vertices shifted by
the extent minimum (``:96-98``).  scikit-image is absent here, so this module
restates the part of that call the reference's test pins -- which grid edges
carry a vertex -- and a table-free polygonisation of its own:

* a cube (lower corner ``p``) is processed when the mask is true at its far
  corner ``p + (1, 1, 1)``;
* every grid edge whose two end values lie on different sides of the level
  (``F > level``) and that belongs to at least one processed cube carries one
  vertex, shared by all cubes around it, placed by linear interpolation;
  vertex ids follow the edge order ``3 * point + axis``;
* a processed cube's polygons are the boundary, on the cube's surface, of its
  ``F <= level`` region: one segment per cube face with two crossings, two
  with four (the pairing chosen by the bilinear saddle value of the face, the
  asymptotic decider of Nielson & Hamann 1991, so both cubes that share the
  face agree), each segment oriented with the ``F <= level`` side on its left
  seen from outside the cube; the linked segments form closed cycles, each
  triangulated as a fan from its first edge.

With these rules the vertex counts of the combination model on a 40x20x20
dense grid are the reference's 600, 860, 1256 and 1680
(``test/test_modules/test_marching_cubes.py:44-47``); ``tests/test_oracle.py``
checks them.  Grid layout: ``field[(i * ny + j) * nz + k]`` (``ij`` order, z
fastest); a vertex on the edge from grid index ``i`` to ``i + 1`` along axis a
sits at ``(i + t) * spacing[a] + origin[a]`` with
``t = (level - F0) / (F1 - F0)``.
"""
import numpy as np

# cube corners: bit 2 = x, bit 1 = y, bit 0 = z
CORNERS = np.array([[(q >> 2) & 1, (q >> 1) & 1, q & 1] for q in range(8)], dtype=np.int64)


def _cube_edges():
    """The 12 cube edges as (axis, start corner, end corner), ids 0-3 along
    x, 4-7 along y, 8-11 along z."""
    out = []
    for a in range(3):
        o = [b for b in range(3) if b != a]
        for hi in (0, 1):
            for lo in (0, 1):
                c = [0, 0, 0]
                c[o[0]], c[o[1]] = hi, lo
                q0 = c[0] * 4 + c[1] * 2 + c[2]
                c[a] = 1
                q1 = c[0] * 4 + c[1] * 2 + c[2]
                out.append((a, q0, q1))
    return out


EDGES = _cube_edges()
_EDGE_OF = {(min(q0, q1), max(q0, q1)): e for e, (_, q0, q1) in enumerate(EDGES)}


def _cube_faces():
    """The 6 faces as (normal axis, side, 4 corners in cyclic (u, v) order
    (0,0) (1,0) (1,1) (0,1), 4 edges c0-c1, c1-c2, c2-c3, c3-c0)."""
    out = []
    for a in range(3):
        u, v = [b for b in range(3) if b != a]
        for s in (0, 1):
            qs = []
            for cu, cv in ((0, 0), (1, 0), (1, 1), (0, 1)):
                c = [0, 0, 0]
                c[a], c[u], c[v] = s, cu, cv
                qs.append(c[0] * 4 + c[1] * 2 + c[2])
            es = [_EDGE_OF[(min(qs[i], qs[(i + 1) % 4]), max(qs[i], qs[(i + 1) % 4]))] for i in range(4)]
            out.append((a, s, qs, es))
    return out


FACES = _cube_faces()
_EDGE_MID = np.array([(CORNERS[q0] + CORNERS[q1]) / 2.0 for _, q0, q1 in EDGES])


def cube_cycles(g):
    """Closed edge cycles of one cube from its 8 corner values ``g = F - level``
    (corner order of ``CORNERS``); each cycle is a list of cube-edge ids."""
    pos = [gi > 0 for gi in g]
    cross = [pos[q0] != pos[q1] for _, q0, q1 in EDGES]
    nxt = [-1] * 12
    for a, s, qs, es in FACES:
        ce = [e for e in es if cross[e]]
        if not ce:
            continue
        normal = np.zeros(3)
        normal[a] = 2 * s - 1
        if len(ce) == 2:
            neg = next(q for q in qs if not pos[q])
            segs = [(ce[0], ce[1], neg)]
        else:
            g0, g1, g2, g3 = (g[q] for q in qs)
            saddle = (g0 * g2 - g1 * g3) / (g0 + g2 - g1 - g3)
            if (saddle > 0) == pos[qs[0]]:
                cut = (1, 3)      # corners 0 and 2 connect through the face centre
            else:
                cut = (0, 2)
            segs = []
            for ci in cut:
                cc = qs[ci]
                e_in, e_out = es[(ci + 3) % 4], es[ci]      # the face edges meeting at corner ci
                neg = cc if not pos[cc] else qs[(ci + 1) % 4]
                segs.append((e_in, e_out, neg))
        for e1, e2, neg in segs:
            d = _EDGE_MID[e2] - _EDGE_MID[e1]
            w = CORNERS[neg] - _EDGE_MID[e1]
            if np.dot(np.cross(d, w), normal) < 0:
                e1, e2 = e2, e1
            nxt[e1] = e2
    cycles, seen = [], [False] * 12
    for e in range(12):
        if cross[e] and not seen[e]:
            cyc = [e]
            seen[e] = True
            f = nxt[e]
            while f != e:
                cyc.append(f)
                seen[f] = True
                f = nxt[f]
            cycles.append(cyc)
    return cycles


def marching_cubes(field, shape, level, spacing=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0), mask=None):
    """(vertices (n_v, 3) float64, faces (n_f, 3) int32) of the level surface."""
    nx, ny, nz = (int(v) for v in shape)
    F = np.asarray(field, dtype=np.float64).reshape(nx, ny, nz)
    M = np.ones((nx, ny, nz), dtype=bool) if mask is None else np.asarray(mask, dtype=bool).reshape(nx, ny, nz)
    level = float(level)
    pos = F > level
    proc = np.zeros((nx, ny, nz), dtype=bool)          # processed cubes by lower corner
    proc[:-1, :-1, :-1] = M[1:, 1:, 1:]
    n = nx * ny * nz
    edge_vid = np.full(3 * n, -1, dtype=np.int64)
    flags = np.zeros((nx, ny, nz, 3), dtype=bool)
    for a in range(3):
        hi = [slice(None)] * 3
        lo = [slice(None)] * 3
        hi[a], lo[a] = slice(1, None), slice(0, -1)
        cr = np.zeros((nx, ny, nz), dtype=bool)
        cr[tuple(lo)] = pos[tuple(lo)] != pos[tuple(hi)]
        used = np.zeros((nx, ny, nz), dtype=bool)
        u, v = [b for b in range(3) if b != a]
        for du in (0, 1):
            for dv in (0, 1):
                sh = [0, 0, 0]
                sh[u], sh[v] = du, dv
                # the cube with lower corner p - sh holds the edge (p, a)
                src = [slice(0, (nx, ny, nz)[b] - sh[b]) for b in range(3)]
                dst = [slice(sh[b], None) for b in range(3)]
                used[tuple(dst)] |= proc[tuple(src)]
        flags[..., a] = cr & used
    fl = flags.reshape(-1)
    idx = np.nonzero(fl)[0]
    edge_vid[idx] = np.arange(len(idx))
    p, a = idx // 3, idx % 3
    ijk = np.stack(np.unravel_index(p, (nx, ny, nz)), axis=1)
    stride = np.array([ny * nz, nz, 1])
    f0 = F.reshape(-1)[p]
    f1 = F.reshape(-1)[p + stride[a]]
    t = (level - f0) / (f1 - f0)
    sp = np.asarray(spacing, dtype=np.float64)
    org = np.asarray(origin, dtype=np.float64)
    verts = ijk.astype(np.float64) * sp + org
    verts[np.arange(len(idx)), a] = (ijk[np.arange(len(idx)), a] + t) * sp[a] + org[a]
    # faces, cube by cube in lower-corner order
    faces = []
    offs = np.array([c[0] * stride[0] + c[1] * stride[1] + c[2] for c in CORNERS])
    Ff = F.reshape(-1)
    for pc in np.nonzero(proc.reshape(-1))[0]:
        g = Ff[pc + offs] - level
        gp = g > 0
        if gp.all() or not gp.any():
            continue
        for cyc in cube_cycles(g):
            vid = [edge_vid[3 * (pc + offs[EDGES[e][1]]) + EDGES[e][0]] for e in cyc]
            for i in range(1, len(vid) - 1):
                faces.append((vid[0], vid[i], vid[i + 1]))
    faces = np.asarray(faces, dtype=np.int32).reshape(-1, 3)
    return verts, faces
