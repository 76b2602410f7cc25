"""MikkTSpace tangents for normal-mapped glTF primitives that carry none.

The reference loader calls the `mikktspace` crate (version 0.3.0, the Rust
port of Morten S. Mikkelsen's reference implementation) through the
Geometry trait in crates/libs/asset_loader/src/geometry.rs:197-212 and
:296-350.  This module restates the published algorithm in numpy, in FP32:

1. vertices with bit-equal position, normal and texture coordinate are
   welded into one vertex (identity for most glTF files);
2. a triangle with two equal positions is degenerate and takes no part in
   steps 3-6;
3. per triangle, the UV-gradient directions vOs (tangent) and vOt
   (bitangent) are normalised and signed by the UV orientation (the sign of
   twice the signed UV area); a triangle without a usable gradient may join
   any group ("group with any");
4. triangles are adjacent across an edge that their welded corners share in
   opposite winding (edges taken in (min index, max index, triangle) order,
   each pairing with the first unpaired candidate);
5. around every welded vertex, the triangles reachable across shared edges
   whose UV orientation agrees form a group (depth-first, left neighbour
   first; a "group with any" triangle takes the orientation of the first
   group that reaches it);
6. per group, each triangle's vOs and vOt are projected into the plane of
   the vertex normal and normalised; triangles whose projected directions
   are not (exactly) opposite share a subgroup (the crate's default angular
   threshold of 180 degrees), and a subgroup's tangent space is the sum over
   its triangles, in index order, of the projected directions weighted by
   the corner angle in that plane, normalised;
7. a corner of a degenerate triangle copies the tangent space of the first
   corner of a healthy triangle with the same welded vertex.

The reference's Geometry::set_tangent stores each face corner's tangent at
its glTF vertex index (the last face that names a vertex wins) with
w = -1 when the corner's group preserves the UV orientation and +1 when it
does not (geometry.rs:333-349), which is the opposite of the crate's own
encoding; that is what the shaders read (RayTracing.rchit:124-127).
Vertices that no face names keep the loader's default (1, 0, 0, 0).
"""
import numpy as np

F = np.float32
FLT_MIN = F(1.17549435e-38)
_ONE = F(1.0)


def _nz(x):
    return np.abs(x) > FLT_MIN


def _vnz(v):
    return np.any(_nz(v), axis=-1)


def _dot(a, b):
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def _normalize_if(v):
    """v / |v| (as v * (1 / |v|)) where any component is non-zero, else v."""
    ln = np.sqrt(_dot(v, v))
    ok = _vnz(v)
    s = np.where(ok, _ONE / np.where(ok, ln, _ONE), _ONE).astype(F)
    return (v * s[..., None]).astype(F)


def _project(v, n):
    """v - dot(n, v) n, normalised where non-zero."""
    return _normalize_if((v - _dot(n, v)[..., None] * n).astype(F))


def _weld(pos, nrm, uv):
    """Welded id of every vertex: the smallest index with bit-equal (after
    +0.0, which makes -0 and +0 equal) position, normal and uv."""
    key = np.concatenate([pos, nrm, uv], 1).astype(F) + F(0.0)
    raw = np.ascontiguousarray(key).view(np.dtype((np.void, key.dtype.itemsize * key.shape[1]))).ravel()
    _, first, inv = np.unique(raw, return_index=True, return_inverse=True)
    return first[inv.ravel()]


def _neighbours(W):
    """nb[f, k]: the triangle across edge k (corner k -> k+1) of triangle f,
    or -1 (step 4)."""
    T = len(W)
    a = W.reshape(-1)
    b = W[:, [1, 2, 0]].reshape(-1)
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    face = np.repeat(np.arange(T), 3)
    order = np.lexsort((face, hi, lo))
    nb = np.full(3 * T, -1, np.int64)
    lo_s, hi_s = lo[order], hi[order]
    start = np.flatnonzero(np.r_[True, (lo_s[1:] != lo_s[:-1]) | (hi_s[1:] != hi_s[:-1])])
    end = np.r_[start[1:], len(order)]
    for s, e in zip(start, end):
        if e - s < 2:
            continue
        run = order[s:e]  # entries f*3+k in (triangle) order
        for x in range(len(run)):
            ea = run[x]
            if nb[ea] >= 0:
                continue
            for y in range(x + 1, len(run)):
                eb = run[y]
                # opposite winding: A's (first, second) is B's (second, first)
                if nb[eb] < 0 and a[ea] == b[eb] and b[ea] == a[eb]:
                    nb[ea], nb[eb] = eb // 3, ea // 3
                    break
    return nb.reshape(T, 3)


def _groups(W, nb, orient, any_):
    """Step 5.  Returns grp[f, k] (group of corner k of triangle f, -1 when
    none), the groups' orientation, their welded vertex and their triangles
    in the order they joined."""
    T = len(W)
    grp = np.full((T, 3), -1, np.int64)
    orient = orient.copy()
    g_orient, g_vert, g_faces = [], [], []
    for f in range(T):
        if any_[f]:
            continue
        for i in range(3):
            if grp[f, i] >= 0:
                continue
            g = len(g_vert)
            v = W[f, i]
            go = bool(orient[f])
            g_orient.append(go)
            g_vert.append(v)
            members = [f]
            grp[f, i] = g
            # depth first, left neighbour (edge i) before right (edge i - 1)
            stack = [x for x in (nb[f, (i + 2) % 3], nb[f, i]) if x >= 0]
            while stack:
                t = stack.pop()
                c = int(np.flatnonzero(W[t] == v)[0])
                if grp[t, c] >= 0:
                    continue
                if any_[t] and np.all(grp[t] < 0):
                    orient[t] = go
                if bool(orient[t]) != go:
                    continue
                members.append(t)
                grp[t, c] = g
                for x in (nb[t, (c + 2) % 3], nb[t, c]):
                    if x >= 0:
                        stack.append(x)
            g_faces.append(members)
    return grp, np.array(g_orient, bool), np.array(g_vert, np.int64), g_faces


def _corner_terms(pos, nrm, W, tri_os, tri_ot, faces, corners, verts):
    """Per (triangle, corner) of a group: the projected vOs, vOt and the
    corner angle in the plane of the vertex normal (step 6)."""
    n = nrm[verts]
    vos = _project(tri_os[faces], n)
    vot = _project(tri_ot[faces], n)
    i0 = W[faces, (corners + 2) % 3]
    i2 = W[faces, (corners + 1) % 3]
    p1 = pos[verts]
    e1 = _project((pos[i0] - p1).astype(F), n)
    e2 = _project((pos[i2] - p1).astype(F), n)
    c = np.clip(_dot(e1, e2), F(-1.0), F(1.0)).astype(F)
    return vos, vot, np.arccos(c).astype(F)


def _eval(vos, ang, use):
    """Angle-weighted sum of the used rows of vos in order, normalised."""
    s = np.zeros(3, F)
    for k in np.flatnonzero(use):
        s = (s + ang[k] * vos[k]).astype(F)
    return _normalize_if(s[None])[0]


def tangents(pos, nrm, uv, tri):
    """Per-vertex tangents (x, y, z, w), float32, as the reference stores
    them for a primitive with positions `pos`, normals `nrm`, texture
    coordinates `uv` (zeros when the primitive has none) and triangles
    `tri` (glTF vertex indices)."""
    pos = np.asarray(pos, F)[:, :3]
    nrm = np.asarray(nrm, F)[:, :3]
    uv = np.asarray(uv, F)[:, :2]
    tri = np.asarray(tri, np.int64).reshape(-1, 3)
    nv, T = len(pos), len(tri)
    out = np.tile(np.array([1, 0, 0, 0], F), (nv, 1))
    if T == 0:
        return out
    weld = _weld(pos, nrm, uv)
    Wall = weld[tri]
    P = pos[Wall]
    degen = (np.all(P[:, 0] == P[:, 1], 1) | np.all(P[:, 0] == P[:, 2], 1) | np.all(P[:, 1] == P[:, 2], 1))
    good = np.flatnonzero(~degen)
    W = Wall[good]

    # step 3
    t = uv[W]
    v = pos[W]
    t21x, t21y = t[:, 1, 0] - t[:, 0, 0], t[:, 1, 1] - t[:, 0, 1]
    t31x, t31y = t[:, 2, 0] - t[:, 0, 0], t[:, 2, 1] - t[:, 0, 1]
    d1, d2 = (v[:, 1] - v[:, 0]).astype(F), (v[:, 2] - v[:, 0]).astype(F)
    area = (t21x * t31y - t21y * t31x).astype(F)
    vos = (t31y[:, None] * d1 - t21y[:, None] * d2).astype(F)
    vot = (-t31x[:, None] * d1 + t21x[:, None] * d2).astype(F)
    orient = area > 0
    los, lot = np.sqrt(_dot(vos, vos)).astype(F), np.sqrt(_dot(vot, vot)).astype(F)
    fs = np.where(orient, F(1.0), F(-1.0)).astype(F)
    ok_a = _nz(area)
    tri_os = np.where((ok_a & _nz(los))[:, None], vos * (fs / np.where(_nz(los), los, _ONE))[:, None], F(0.0)).astype(F)
    tri_ot = np.where((ok_a & _nz(lot))[:, None], vot * (fs / np.where(_nz(lot), lot, _ONE))[:, None], F(0.0)).astype(F)
    absa = np.where(ok_a, np.abs(area), _ONE)
    any_ = ~(ok_a & _nz(los / absa) & _nz(lot / absa))

    # steps 4-5
    nb = _neighbours(W)
    grp, g_orient, g_vert, g_faces = _groups(W, nb, orient, any_)

    # step 6: subgroups and their tangent spaces, over every (group, triangle) pair at once
    ts_os = np.tile(np.array([1, 0, 0], F), (len(good), 3, 1))
    ts_or = np.zeros((len(good), 3), bool)
    if g_faces:
        sizes = np.array([len(m) for m in g_faces], np.int64)
        pg = np.repeat(np.arange(len(g_faces)), sizes)
        pf = np.concatenate([np.array(m, np.int64) for m in g_faces])
        pv = g_vert[pg]
        pc = np.argmax(W[pf] == pv[:, None], axis=1)
        p_os, p_ot, ang = _corner_terms(pos, nrm, W, tri_os, tri_ot, pf, pc, pv)
        # every ordered pair (r, q) of rows of the same group
        off = np.r_[0, np.cumsum(sizes)[:-1]]
        rr = np.repeat(np.arange(len(pf)), sizes[pg])
        qq = off[pg[rr]] + (np.arange(len(rr)) - np.repeat(np.r_[0, np.cumsum(sizes[pg])[:-1]], sizes[pg]))
        joined = (any_[pf[rr]] | any_[pf[qq]] | (rr == qq) |
                  ((_dot(p_os[rr], p_os[qq]) > F(-1.0)) & (_dot(p_ot[rr], p_ot[qq]) > F(-1.0))))
        split = np.zeros(len(g_faces), bool)
        split[pg[rr[~joined]]] = True
        # groups whose triangles all join: one subgroup, summed in triangle order
        order = np.lexsort((pf, pg))
        use = order[~split[pg[order]] & ~any_[pf[order]]]
        acc = np.zeros((len(g_faces), 3), F)
        np.add.at(acc, pg[use], (ang[use, None] * p_os[use]).astype(F))
        g_ts = _normalize_if(acc)
        whole = ~split[pg]
        ts_os[pf[whole], pc[whole]] = g_ts[pg[whole]]
        ts_or[pf, pc] = g_orient[pg]
        # groups with (exactly) opposite projected directions: a subgroup per distinct member set
        for g in np.flatnonzero(split):
            rows = np.flatnonzero(pg == g)
            cache = {}
            for r in rows:
                sel = np.sort(pf[qq[(rr == r) & joined]])
                key = sel.tobytes()
                if key not in cache:
                    o = rows[np.argsort(pf[rows])]
                    u = np.isin(pf[o], sel) & ~any_[pf[o]]
                    cache[key] = _eval(p_os[o], ang[o], u)
                ts_os[pf[r], pc[r]] = cache[key]

    # step 7 and the per-face-corner output in face order
    full_os = np.tile(np.array([1, 0, 0], F), (T, 3, 1))
    full_or = np.zeros((T, 3), bool)
    full_os[good], full_or[good] = ts_os, ts_or
    bad = np.flatnonzero(degen)
    if len(bad):
        flat = W.reshape(-1)
        ids, first = np.unique(flat, return_index=True)
        for f in bad:
            for c in range(3):
                k = np.searchsorted(ids, Wall[f, c])
                if k < len(ids) and ids[k] == Wall[f, c]:
                    j = first[k]
                    full_os[f, c] = ts_os[j // 3, j % 3]
                    full_or[f, c] = ts_or[j // 3, j % 3]
    vals = np.concatenate([full_os.reshape(-1, 3), np.where(full_or.reshape(-1, 1), F(-1.0), F(1.0))], 1)
    idx = tri.reshape(-1)
    rev = idx[::-1]
    u, first_rev = np.unique(rev, return_index=True)
    out[u] = vals[len(idx) - 1 - first_rev]
    return out.astype(F)
