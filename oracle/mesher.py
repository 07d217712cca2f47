"""CPU restatement of the reference's surface mesher (getIsomesh), in numpy.

TEST INFRASTRUCTURE: only tests/ use it, as the checker of the library's
GPU mesher; it is never the product path.  It restates what the reference
does at the first substep of a frame (FluidSimulation::_outputSurfaceMeshThread,
src/engine/fluidsimulation.cpp:5150-5219), step by step:

  * ParticleMesher (particlemesher.cpp): active blocks of 10^3 nodes and
    their 26-neighbour feathering (:116-137, gridutils.cpp:265-298); the one
    compute chunk (:139-282); the block lists of the count pass (:400-446)
    and the per-block distance minimum (:498-549); negation (:472-478);
  * ScalarField's solid vertices (scalarfield.cpp:372-448,
    meshlevelset.cpp:291-340) and Interpolation::trilinearInterpolate
    (interpolation.cpp:61-113);
  * Polygonizer3d (polygonizer3d.cpp:356-675): cube indices, vertex
    interpolation kept off the solid, the order vertices are created in,
    the triangle table;
  * TriangleMesh::smooth (trianglemesh.cpp:481-585).

Parity pin: tests/test_surface.py checks this restatement against the
fixtures tests/golden/make_golden.py made from the reference itself
(iso_*.npz), bit for bit.
"""
from __future__ import annotations

import numpy as np

f32, f64 = np.float32, np.float64
MB = 10   # ParticleMesher::_blockwidth

# The published marching-cubes triangle table (Lorensen and Cline's cases
# as Paul Bourke tabulated them; polygonizer3d.cpp:97-354 holds the same):
# case q's edge ids in the 4-bit fields of TRI[q], lowest first, 0xF ends.
TRI = [
    0xffffffffffffffff, 0xfffffffffffff380, 0xfffffffffffff910, 0xffffffffff189381,
    0xfffffffffffffa21, 0xffffffffffa21380, 0xffffffffff920a29, 0xfffffff89a8a2382,
    0xfffffffffffff2b3, 0xffffffffff0b82b0, 0xffffffffffb32091, 0xfffffffb89b912b1,
    0xffffffffff3ab1a3, 0xfffffffab8a801a0, 0xfffffff9ab9b3093, 0xffffffffffb8aa89,
    0xfffffffffffff874, 0xffffffffff437034, 0xffffffffff748910, 0xfffffff137174914,
    0xffffffffff748a21, 0xfffffffa21403743, 0xfffffff748209a29, 0xffff4973727929a2,
    0xffffffffff2b3748, 0xfffffff40242b74b, 0xfffffffb32748109, 0xffff1292b9b49b74,
    0xfffffff487ab31a3, 0xffff4b7401b41ab1, 0xffff30bab9b09874, 0xfffffffab99b4b74,
    0xfffffffffffff459, 0xffffffffff380459, 0xffffffffff051450, 0xfffffff513538458,
    0xffffffffff459a21, 0xfffffff594a21803, 0xfffffff204245a25, 0xffff8434535235a2,
    0xffffffffffb32459, 0xfffffff594b802b0, 0xfffffffb32510450, 0xffff584b82852512,
    0xfffffff45931ab3a, 0xffffab81a8180594, 0xffff30bab5b05045, 0xfffffffb8aa85845,
    0xffffffffff975879, 0xfffffff375359039, 0xfffffff751710870, 0xffffffffff753351,
    0xfffffff21a759879, 0xffff37503505921a, 0xffff25a758528208, 0xfffffff7533525a2,
    0xfffffff2b3987597, 0xffffb72029279759, 0xffff751871810b32, 0xfffffff51771b12b,
    0xffffb3a31a758859, 0xf0aba010b7905075, 0xf07570805a30b0ab, 0xffffffffff5b75ab,
    0xfffffffffffff56a, 0xffffffffff6a5380, 0xffffffffff6a5109, 0xfffffff6a5891381,
    0xffffffffff162561, 0xfffffff803621561, 0xfffffff620609569, 0xffff823625285895,
    0xffffffffff56ab32, 0xfffffff56a02b80b, 0xfffffff6a5b32910, 0xffffb892b92916a5,
    0xfffffff315356b36, 0xffff6b51505b0b80, 0xffff9505606306b3, 0xfffffff89bb96956,
    0xffffffffff8746a5, 0xfffffffa56374034, 0xfffffff7486a5091, 0xffff49737179156a,
    0xfffffff874156216, 0xffff743403625521, 0xffff620560509748, 0xf962695923497937,
    0xfffffff56a4872b3, 0xffffb720242746a5, 0xffff6a5b32874910, 0xf6a54b7b492b9129,
    0xffff6b51535b3748, 0xfb404b7b016b5b15, 0xf74836b630560950, 0xffff9b7974b96956,
    0xffffffffffa4694a, 0xfffffff380a946a4, 0xfffffff04606a10a, 0xffffa16468618138,
    0xfffffff462421941, 0xffff462942921803, 0xffffffffff624420, 0xfffffff624428238,
    0xfffffff32b46a94a, 0xffff6a4a94b82280, 0xffffa164606102b3, 0xf1b8b12184a16146,
    0xffff36b319639469, 0xf14641916b0181b8, 0xfffffff4600636b3, 0xffffffffff86b846,
    0xfffffffa98a876a7, 0xffffa76a907a0370, 0xffff0818717a176a, 0xfffffff37117a76a,
    0xffff768981861621, 0xf937390976192962, 0xfffffff206607087, 0xffffffffff276237,
    0xffff76898a86ab32, 0xf7a9a76790b72702, 0xfb32a767a1871081, 0xffff17616a71b12b,
    0xf63136b619768698, 0xffffffffff76b190, 0xffff06b0b3607087, 0xfffffffffffff6b7,
    0xfffffffffffffb67, 0xffffffffff67b803, 0xffffffffff67b910, 0xfffffff67b138918,
    0xffffffffff7b621a, 0xfffffff7b6803a21, 0xfffffff7b69a2092, 0xffff89a38a3a27b6,
    0xffffffffff726327, 0xfffffff026067807, 0xfffffff910732672, 0xffff678891681261,
    0xfffffff73171a67a, 0xffff801781a7167a, 0xffff7a69a0a70730, 0xfffffff9a88a7a67,
    0xffffffffff68b486, 0xfffffff640603b63, 0xfffffff109648b68, 0xffff63b139369649,
    0xfffffff1a28b6486, 0xffff640b60b03a21, 0xffff9a2920b648b4, 0xf36463b34923a39a,
    0xfffffff264248328, 0xffffffffff264240, 0xffff834642432091, 0xfffffff642241491,
    0xffff1a6648168318, 0xfffffff40660a01a, 0xf39a9303a6834364, 0xffffffffff4a649a,
    0xffffffffffb67594, 0xfffffff67b594380, 0xfffffffb67045105, 0xffff51345343867b,
    0xfffffffb6721a459, 0xffff594380a217b6, 0xffff204a24a45b67, 0xf67b25a523453843,
    0xfffffff945267327, 0xffff786260680459, 0xffff045051673263, 0xf851584812786826,
    0xffff73167161a459, 0xf459078701671a61, 0xfa737a6a305a4a04, 0xffffa84a458a7a67,
    0xfffffff98b9b6596, 0xffff590650360b63, 0xffffb65510b508b0, 0xfffffff1355363b6,
    0xffff65b8b9b59a21, 0xfa21965690b603b0, 0xf52025a50865b58b, 0xffff35a3a25363b6,
    0xffff283265825985, 0xfffffff260069659, 0xf826283865081851, 0xffffffffff612651,
    0xf698965683a61631, 0xffff06505960a01a, 0xffffffffffa65830, 0xfffffffffffff65a,
    0xffffffffffb57a5b, 0xfffffff03857ba5b, 0xfffffff091ba57b5, 0xffff1381897ba57a,
    0xfffffff15717b21b, 0xffffb27571721380, 0xffff7b2209729579, 0xf289823295b27257,
    0xfffffff573532a52, 0xffff52a578258028, 0xffff2a37353a5109, 0xf25752a278129289,
    0xffffffffff573531, 0xfffffff571170780, 0xfffffff735539309, 0xffffffffff795789,
    0xfffffff8ba8a5485, 0xffff03bba50b5405, 0xffff54aba8a48910, 0xf41314943b54a4ba,
    0xffff8548b2582152, 0xfb151b2b543b0b40, 0xf58b8545b2950520, 0xffffffffff3b2549,
    0xffff483543253a52, 0xfffffff0244252a5, 0xf910854583a532a3, 0xffff2492914252a5,
    0xfffffff153358548, 0xffffffffff501540, 0xffff530509358548, 0xfffffffffffff549,
    0xfffffffba9b947b4, 0xffffba97b9794380, 0xffffb470414b1ba1, 0xf4bab474a1843413,
    0xffff219b294b97b4, 0xf3801b2b197b9479, 0xfffffff04224b47b, 0xffff42343824b47b,
    0xffff947732972a92, 0xf70207872a4797a9, 0xfa040a1a472a3a73, 0xffffffffff4782a1,
    0xfffffff317714194, 0xffff178180714194, 0xffffffffff347304, 0xfffffffffffff784,
    0xffffffffff8ba8a9, 0xfffffffa9bb93903, 0xfffffffba88a0a10, 0xffffffffffa3ba13,
    0xfffffff8b99b1b21, 0xffff9b2921b93903, 0xffffffffffb08b20, 0xfffffffffffffb23,
    0xfffffff98aa82832, 0xffffffffff2902a9, 0xffff8a1810a82832, 0xfffffffffffff2a1,
    0xffffffffff819831, 0xfffffffffffff190, 0xfffffffffffff830, 0xffffffffffffffff,]
# cube corners (grid3d.h:304-313) and edges in the reference's order
# (polygonizer3d.cpp:495-630): corners interpolated from/to, axis, and the
# corner the edge starts from along its axis
CX = np.array([0, 1, 1, 0, 0, 1, 1, 0])
CY = np.array([0, 0, 0, 0, 1, 1, 1, 1])
CZ = np.array([0, 0, 1, 1, 0, 0, 1, 1])
EA = [0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3]
EB = [1, 2, 3, 0, 5, 6, 7, 4, 4, 5, 6, 7]
EDIR = [0, 2, 0, 2, 0, 2, 0, 2, 1, 1, 1, 1]
EORG = [0, 1, 3, 0, 4, 5, 7, 4, 0, 1, 2, 3]


def _tri_edges(q):
    w, out = TRI[q], []
    for t in range(16):
        e = (w >> (4 * t)) & 0xF
        if e == 0xF:
            break
        out.append(e)
    return out


TRI_EDGES = [_tri_edges(q) for q in range(256)]
NTRI = np.array([len(t) // 3 for t in TRI_EDGES])
CUT = np.array([sum(1 << e for e in range(12) if ((q >> EA[e]) ^ (q >> EB[e])) & 1) for q in range(256)])


def _floor_idx(p32, inv):
    """Grid3d::positionToGridIndex: floor((double)p * inv)."""
    return np.floor(np.asarray(p32, f32).astype(f64) * inv).astype(np.int64)


def _idx_pos(i, dx):
    """Grid3d::GridIndexToPosition: (float)((double)(float)i * dx)."""
    return (np.asarray(i).astype(f32).astype(f64) * dx).astype(f32)


def trilinear(phi, dx, p):
    """Interpolation::trilinearInterpolate(vec3 p, dx, grid) in FP64 on the
    nodal grid phi (k, j, i); p: (n, 3) float32."""
    p = np.asarray(p, f32)
    inv = 1.0 / dx
    g = _floor_idx(p, inv)
    gpos = _idx_pos(g, dx)
    x = (p - gpos).astype(f32).astype(f64) * inv
    nk, nj, ni = phi.shape

    def at(di, dj, dk):
        a, b, c = g[:, 0] + di, g[:, 1] + dj, g[:, 2] + dk
        ok = (a >= 0) & (b >= 0) & (c >= 0) & (a < ni) & (b < nj) & (c < nk)
        out = np.zeros(len(p), f64)
        out[ok] = phi[c[ok], b[ok], a[ok]]
        return out

    X, Y, Z = x[:, 0], x[:, 1], x[:, 2]
    return (at(0, 0, 0) * (1 - X) * (1 - Y) * (1 - Z) + at(1, 0, 0) * X * (1 - Y) * (1 - Z) +
            at(0, 1, 0) * (1 - X) * Y * (1 - Z) + at(0, 0, 1) * (1 - X) * (1 - Y) * Z +
            at(1, 0, 1) * X * (1 - Y) * Z + at(0, 1, 1) * (1 - X) * Y * Z + at(1, 1, 0) * X * Y * (1 - Z) +
            at(1, 1, 1) * X * Y * Z)


def mesh_particles(pos, isize, jsize, ksize, dx, solid_phi, subdivisions=1, particle_scale=3.0,
                   smooth_value=0.5, smooth_iterations=2):
    """The reference's isomesh of the particles `pos` ((n, 3) float32) on an
    isize x jsize x ksize grid of cell size dx with the nodal solid level set
    solid_phi ((k+1, j+1, i+1) float32).  Returns (vertices (m, 3) float32,
    triangles (t, 3) int32)."""
    pos = np.ascontiguousarray(pos, f32)
    empty = (np.zeros((0, 3), f32), np.zeros((0, 3), np.int32))
    if len(pos) == 0:
        return empty
    I, J, K = isize, jsize, ksize
    sd = subdivisions
    subdx = dx / sd
    volume = dx * dx * dx / 8.0
    radius = (3 * volume / (4 * 3.141592653)) ** (1.0 / 3.0) * particle_scale
    r = f32(radius)
    sr = f32(f32(1.5) * r)
    maxd = f32(3.0 * radius)
    sub = np.array([I * sd + 1, J * sd + 1, K * sd + 1])
    nb = (sub + MB - 1) // MB
    # active blocks, feathered
    occ = np.zeros(nb[::-1], bool)
    b = _floor_idx(pos, 1.0 / (MB * subdx))
    occ[b[:, 2], b[:, 1], b[:, 0]] = True
    act = occ.copy()
    for dk in (-1, 0, 1):
        for dj in (-1, 0, 1):
            for di in (-1, 0, 1):
                src = occ[max(-dk, 0):nb[2] - max(dk, 0), max(-dj, 0):nb[1] - max(dj, 0), max(-di, 0):nb[0] - max(di, 0)]
                act[max(dk, 0):nb[2] - max(-dk, 0), max(dj, 0):nb[1] - max(-dj, 0), max(di, 0):nb[0] - max(-di, 0)] |= src
    if not act.any():
        return empty
    kk, jj, ii = np.nonzero(act)
    lo = np.array([ii.min(), jj.min(), kk.min()])
    hi = np.array([ii.max(), jj.max(), kk.max()]) + 1
    split = 0
    if nb[1] > nb[0]:
        split = 1
    if nb[2] > nb[split]:
        split = 2
    for d in range(3):
        if d != split:
            lo[d] = max(lo[d] - 1, 0)
            hi[d] = min(hi[d] + 1, nb[d])
    gmin = MB * lo
    gmax = np.minimum(MB * hi, sub)
    nn = gmax - gmin                       # chunk nodes (i, j, k)
    off = _idx_pos(gmin, subdx)            # chunk offset (float)
    cb = hi - lo
    cact = act[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]]
    # the chunk's box, expanded (aabb.cpp:40-52, 122-133)
    pmax = _idx_pos(gmax, subdx)
    v = 2.0 * (radius + float(f32(1e-6)))
    h = 0.5 * v
    bpos = (off - f32(h)).astype(f32)
    bsize = (pmax.astype(f64) - off.astype(f64)) + v
    inside = np.all(pos >= bpos, axis=1) & np.all(pos.astype(f64) < bpos.astype(f64) + bsize, axis=1)
    pc = (pos[inside] - off).astype(f32)
    # the count pass's block lists
    bdxF = f32(MB * subdx)
    invF = 1.0 / float(bdxF)
    own = _floor_idx(pc, invF)
    bp = (own.astype(f32).astype(f64) * float(bdxF)).astype(f32)
    simple = (np.all((pc - sr).astype(f32) > bp, axis=1) &
              np.all((pc + sr).astype(f32) < (bp + bdxF).astype(f32), axis=1))
    b0 = np.where(simple[:, None], own, _floor_idx((pc - sr).astype(f32), invF))
    b1 = np.where(simple[:, None], own, _floor_idx((pc + sr).astype(f32), invF))
    best = np.full(nn[::-1], np.inf, f32)   # smallest squared distance per chunk node (k, j, i)
    npos = _idx_pos(np.arange(MB), subdx)
    invs = 1.0 / subdx
    for dk in (0, 1):
        for dj in (0, 1):
            for di in (0, 1):
                B = b0 + np.array([di, dj, dk])
                ok = np.all(B <= b1, axis=1) & np.all(B >= 0, axis=1) & np.all(B < cb, axis=1)
                ok[ok] &= cact[B[ok, 2], B[ok, 1], B[ok, 0]]
                if not ok.any():
                    continue
                Bq = B[ok]
                boff = (Bq.astype(f32).astype(f64) * (MB * subdx)).astype(f32)
                loc = (pc[ok] - boff).astype(f32)
                a0 = np.maximum(_floor_idx((loc - sr).astype(f32), invs), 0)
                a1 = np.minimum(_floor_idx((loc + sr).astype(f32), invs) + 1, MB - 1)
                span = int((a1 - a0).max()) + 1
                for oz in range(span):
                    for oy in range(span):
                        for ox in range(span):
                            a = a0 + np.array([ox, oy, oz])
                            m = np.all(a <= a1, axis=1)
                            if not m.any():
                                continue
                            am, lm, bm = a[m], loc[m], Bq[m]
                            d = (npos[am] - lm).astype(f32)
                            d2 = ((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]).astype(f32) + d[:, 2] * d[:, 2]).astype(f32)
                            g = MB * bm + am
                            sel = np.all(g < nn, axis=1)
                            np.minimum.at(best, (g[sel, 2], g[sel, 1], g[sel, 0]), d2[sel])
    with np.errstate(invalid="ignore"):
        dist = np.where(np.isinf(best), maxd, np.minimum(maxd, (np.sqrt(best).astype(f32) - r).astype(f32)))
    field = (-dist).astype(f32)
    # solid vertices clamp to the surface threshold (scalarfield.cpp:372-448)
    kc, jc, ic = np.nonzero(field > 0)
    if len(ic):
        same = (tuple(nn) == (I + 1, J + 1, K + 1)) and abs(subdx - dx) < 1e-12
        aligned = abs(2 * subdx - dx) < 1e-6 and float(np.sqrt(f32(off @ off))) < 1e-6
        if same:
            solid = solid_phi[kc, jc, ic] < 0
        else:
            q = np.stack([ic, jc, kc], 1)
            p = (_idx_pos(q, subdx) + off).astype(f32)
            d = trilinear(solid_phi, dx, p)
            solid = (d.astype(f32) < 0) if aligned else (d < 0)
            if aligned:
                even = np.all(q % 2 == 0, axis=1)
                solid[even] = solid_phi[kc[even] // 2, jc[even] // 2, ic[even] // 2] < 0
        field[kc[solid], jc[solid], ic[solid]] = 0.0
    # cube indices, new vertices and triangles per cell, in flat order
    ci, cj, ck = nn - 1
    if ci <= 0 or cj <= 0 or ck <= 0:
        return empty
    cube = np.zeros((ck, cj, ci), np.int64)
    for q in range(8):
        cube |= (field[CZ[q]:CZ[q] + ck, CY[q]:CY[q] + cj, CX[q]:CX[q] + ci] > 0).astype(np.int64) << q
    kz, jy, ix = np.meshgrid(np.arange(ck), np.arange(cj), np.arange(ci), indexing="ij")

    def created(i, j, k):
        m = 0
        for e in range(12):
            o, d = EORG[e], EDIR[e]
            ok = ((d == 0) | (CX[o] == 1) | (i == 0)) & ((d == 1) | (CY[o] == 1) | (j == 0)) & \
                 ((d == 2) | (CZ[o] == 1) | (k == 0))
            m = m | (ok.astype(np.int64) << e)
        return m

    surf = (cube != 0) & (cube != 255)
    newmask = np.where(surf, CUT[cube] & created(ix, jy, kz), 0)
    nvc = np.zeros_like(newmask)
    for e in range(12):
        nvc += (newmask >> e) & 1
    ntc = np.where(surf, NTRI[cube], 0)
    vstart = (np.cumsum(nvc.ravel()) - nvc.ravel()).reshape(nvc.shape)
    tstart = (np.cumsum(ntc.ravel()) - ntc.ravel()).reshape(ntc.shape)
    nverts, ntris = int(nvc.sum()), int(ntc.sum())
    verts = np.zeros((nverts, 3), f32)
    sdxf = f32(subdx)
    for e in range(12):
        has = (newmask >> e) & 1 == 1
        if not has.any():
            continue
        rank = np.zeros_like(newmask)
        for e2 in range(e):
            rank += (newmask >> e2) & 1
        vi = (vstart + rank)[has]
        k0, j0, i0 = kz[has], jy[has], ix[has]
        A, Bc = EA[e], EB[e]
        pa = np.stack([i0 + CX[A], j0 + CY[A], k0 + CZ[A]], 1)
        pb = np.stack([i0 + CX[Bc], j0 + CY[Bc], k0 + CZ[Bc]], 1)
        p1 = (sdxf * pa.astype(f32)).astype(f32)
        p2 = (sdxf * pb.astype(f32)).astype(f32)
        v1 = field[pa[:, 2], pa[:, 1], pa[:, 0]].astype(f64)
        v2 = field[pb[:, 2], pb[:, 1], pb[:, 0]].astype(f64)
        # Polygonizer3d::_vertexInterp (polygonizer3d.cpp:455-491)
        s1 = trilinear(solid_phi, dx, (p1 + off).astype(f32)).astype(f32).astype(f64)
        s2 = trilinear(solid_phi, dx, (p2 + off).astype(f32)).astype(f32).astype(f64)
        eps = 1e-10
        minmu = np.zeros(len(vi))
        maxmu = np.ones(len(vi))
        cross = ((s1 < 0) & (s2 >= 0)) | ((s2 < 0) & (s1 >= 0))
        diff = s2 - s1
        big = cross & (np.abs(diff) > eps)
        with np.errstate(divide="ignore", invalid="ignore"):
            su = -s1 / diff
        minmu = np.where(big & (s1 < 0), su, minmu)
        maxmu = np.where(big & ~(s1 < 0), su, maxmu)
        maxmu = np.where(cross & ~big, minmu, maxmu)
        minmu = np.maximum(minmu, eps)
        maxmu = np.minimum(maxmu, 1.0 - eps)
        mu = (0.0 - v1) / (v2 - v1)
        mu = np.where(mu < minmu, minmu, mu)
        mu = np.where(mu > maxmu, maxmu, mu)
        fm = mu.astype(f32)[:, None]
        pv = (p1 + (fm * (p2 - p1).astype(f32)).astype(f32)).astype(f32)
        # translate by the chunk offset, scale and unscale (particlemesher.cpp:35-55)
        scale = 0.1 / subdx
        pv = (((pv + off).astype(f32) * f32(scale)).astype(f32) * f32(1.0 / scale)).astype(f32)
        verts[vi] = pv
    # triangles: the vertex of an edge is made by the first cell holding it
    tris = np.zeros((ntris, 3), np.int32)
    cflat = np.nonzero(surf.ravel())[0]
    cubes = cube.ravel()[cflat]
    cidx = np.stack([ix.ravel()[cflat], jy.ravel()[cflat], kz.ravel()[cflat]], 1)
    tbase = tstart.ravel()[cflat]
    lookup = {}
    for e in range(12):
        lookup[(EDIR[e], CX[EORG[e]], CY[EORG[e]], CZ[EORG[e]])] = e

    def edge_vertex(cells, e):
        o, d = EORG[e], EDIR[e]
        n = cells + np.array([CX[o], CY[o], CZ[o]])
        pc2 = n.copy()
        for ax in range(3):
            if ax != d:
                pc2[:, ax] = np.maximum(n[:, ax] - 1, 0)
        offs = n - pc2
        out = np.zeros(len(cells), np.int64)
        for key_o in {(int(x), int(y), int(z)) for x, y, z in offs}:
            sel = np.all(offs == np.array(key_o), axis=1)
            e2 = lookup[(d,) + key_o]
            c2 = pc2[sel]
            mk = newmask[c2[:, 2], c2[:, 1], c2[:, 0]]
            rank = np.zeros(len(c2), np.int64)
            for e3 in range(e2):
                rank += (mk >> e3) & 1
            out[sel] = vstart[c2[:, 2], c2[:, 1], c2[:, 0]] + rank
        return out

    for t in range(5):
        has = NTRI[cubes] > t
        if not has.any():
            continue
        for corner in range(3):
            col = np.zeros(has.sum(), np.int64)
            edges = np.array([TRI_EDGES[q][3 * t + corner] for q in cubes[has]])
            for e in range(12):
                sel = edges == e
                if sel.any():
                    col[sel] = edge_vertex(cidx[has][sel], e)
            tris[tbase[has] + t, corner] = col
    # TriangleMesh::smooth: each vertex's triangles in ascending order
    if smooth_iterations > 0 and ntris > 0:
        vt = np.repeat(np.arange(ntris), 3)
        vv = tris.ravel()
        order = np.lexsort((vt, vv))
        vv, vt = vv[order], vt[order]
        starts = np.searchsorted(vv, np.arange(nverts + 1))
        deg = np.diff(starts)
        value = f32(smooth_value)
        for _ in range(smooth_iterations):
            acc = np.zeros((nverts, 3), f32)
            cnt = np.zeros(nverts, np.int64)
            for slot in range(int(deg.max())):
                has = deg > slot
                v_ids = np.nonzero(has)[0]
                tri = tris[vt[starts[v_ids] + slot]]
                for corner in range(3):
                    u = tri[:, corner]
                    other = u != v_ids
                    acc[v_ids[other]] = (acc[v_ids[other]] + verts[u[other]]).astype(f32)
                    cnt[v_ids[other]] += 1
            inv = (1.0 / cnt.astype(f32).astype(f64)).astype(f32)
            avg = (acc * inv[:, None]).astype(f32)
            verts = (verts + (value * (avg - verts).astype(f32)).astype(f32)).astype(f32)
    return verts, tris
