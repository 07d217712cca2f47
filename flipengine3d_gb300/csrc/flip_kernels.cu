// FLIP step kernels for GB300 (sm_103a): particle binning, liquid SDF, P2G,
// extrapolation, body force, constrain, and the fused PIC/FLIP + RK3 +
// collision particle update.  Every kernel is an HBM-bound gather/stencil;
// nothing here is a dense contraction, so no tensor cores are involved.
#include <cstdio>

#include "flip_device.cuh"

namespace flip {

namespace {

constexpr int TPB = 256;

struct F3 { float x, y, z; };
__device__ __forceinline__ F3 f3(float x, float y, float z) { F3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ F3 add(F3 a, F3 b) { return f3(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)); }
__device__ __forceinline__ F3 sub(F3 a, F3 b) { return f3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)); }
__device__ __forceinline__ F3 mul(float s, F3 v) { return f3(__fmul_rn(v.x, s), __fmul_rn(v.y, s), __fmul_rn(v.z, s)); }
__device__ __forceinline__ float dot3(F3 a, F3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ float len3(F3 a) { return __fsqrt_rn(dot3(a, a)); }
// vmath operator/ : multiply by (float)(1.0 / s)  (src/engine/vmath.cpp:100-103)
__device__ __forceinline__ F3 normalize3(F3 v) {
    float inv = (float)(1.0 / (double)len3(v));
    return mul(inv, v);
}

// ------------------------------------------------------------------ binning
__global__ void k_keys(ParticleSoA p, int n, StepConsts c, unsigned int *keys) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i = exact_floor(p.px[t], c.invdx, c.invdxf);
    int j = exact_floor(p.py[t], c.invdx, c.invdxf);
    int k = exact_floor(p.pz[t], c.invdx, c.invdxf);
    Dims d{c.I, c.J, c.K};
    keys[t] = d.in(i, j, k) ? (unsigned int)d.idx(i, j, k) : KEY_SOLID;
}

__global__ void k_bin_count(const unsigned int *keys, int n, int *count) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    unsigned int k = keys[t];
    if (k & KEY_SOLID) return;
    atomicAdd(&count[k & KEY_CELL_MASK], 1);
}

// Exclusive scan of n ints: 4096 per block, then the block totals.
constexpr int SCAN_T = 1024, SCAN_PER = 4, SCAN_TILE = SCAN_T * SCAN_PER;

__device__ int block_scan_excl(int v, int *sh, int *total) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        sh[lane] = w;
    }
    __syncthreads();
    int base = warp > 0 ? sh[warp - 1] : 0;
    if (total) *total = sh[(blockDim.x >> 5) - 1];
    int r = base + x - v;
    __syncthreads();
    return r;
}

__global__ void k_scan_tiles(const int *in, int n, int *out, int *tileSums) {
    __shared__ int sh[32];
    long long base = (long long)blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER;
    int v[SCAN_PER];
    int sum = 0;
#pragma unroll
    for (int q = 0; q < SCAN_PER; q++) {
        long long g = base + q;
        v[q] = g < n ? in[g] : 0;
        sum += v[q];
    }
    int total;
    int ex = block_scan_excl(sum, sh, &total);
#pragma unroll
    for (int q = 0; q < SCAN_PER; q++) {
        long long g = base + q;
        if (g < n) out[g] = ex;
        ex += v[q];
    }
    if (threadIdx.x == 0) tileSums[blockIdx.x] = total;
}

__global__ void k_scan_sums(int *tileSums, int ntiles, int *grandTotal) {
    __shared__ int sh[32];
    int v[SCAN_PER];
    int sum = 0;
#pragma unroll
    for (int q = 0; q < SCAN_PER; q++) {
        int g = threadIdx.x * SCAN_PER + q;
        v[q] = g < ntiles ? tileSums[g] : 0;
        sum += v[q];
    }
    int total;
    int ex = block_scan_excl(sum, sh, &total);
#pragma unroll
    for (int q = 0; q < SCAN_PER; q++) {
        int g = threadIdx.x * SCAN_PER + q;
        if (g < ntiles) tileSums[g] = ex;
        ex += v[q];
    }
    if (threadIdx.x == 0) *grandTotal = total;
}

__global__ void k_scan_add(int *out, int n, const int *tileSums, const int *grandTotal) {
    long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g < n) out[g] += tileSums[g / SCAN_TILE];
    if (g == n) out[n] = *grandTotal;
}

__global__ void k_bin_scatter(const unsigned int *keys, int n, const int *start, int *cursor, int *slots) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    unsigned int k = keys[t];
    if (k & KEY_SOLID) return;
    int c = (int)(k & KEY_CELL_MASK);
    int pos = start[c] + atomicAdd(&cursor[c], 1);
    slots[pos] = t;
}

// Per cell: order the slots by particle id (the reference's order), then
// apply the 250-per-cell limit (first by id) and the extreme-speed removal,
// as _removeMarkerParticles does (src/engine/fluidsimulation.cpp:4324-4353).
// Kept slots are compacted to the front of the cell's segment.
__global__ void k_cell_sort_select(const int *start, int ncells, int *slots, const unsigned int *ids,
                                   const unsigned int *keys, int maxPerCell, int *survivors) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    int b = start[c], e = start[c + 1];
    for (int a = b + 1; a < e; a++) {
        int s = slots[a];
        unsigned int key = ids[s];
        int q = a - 1;
        while (q >= b && ids[slots[q]] > key) {
            slots[q + 1] = slots[q];
            q--;
        }
        slots[q + 1] = s;
    }
    int kept = 0;
    for (int a = b; a < e; a++) {
        int s = slots[a];
        int rank = a - b;
        if (rank >= maxPerCell) continue;
        if (keys[s] & KEY_FAST) continue;
        slots[b + kept] = s;
        kept++;
    }
    survivors[c] = kept;
}

__global__ void k_gather(ParticleSoA src, ParticleSoA dst, const int *start, const int *slots,
                         const int *newStart, int ncells, unsigned int *maxSpeedSqBits) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    float best = 0.0f;
    if (c < ncells) {
        int b = start[c];
        int o = newStart[c], e = newStart[c + 1];
        for (int q = 0; q < e - o; q++) {
            int s = slots[b + q];
            float vx = src.vx[s], vy = src.vy[s], vz = src.vz[s];
            dst.px[o + q] = src.px[s];
            dst.py[o + q] = src.py[s];
            dst.pz[o + q] = src.pz[s];
            dst.vx[o + q] = vx;
            dst.vy[o + q] = vy;
            dst.vz[o + q] = vz;
            dst.id[o + q] = src.id[s];
            float sq = __fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)), __fmul_rn(vz, vz));
            best = fmaxf(best, sq);
        }
    }
    for (int o = 16; o > 0; o >>= 1) best = fmaxf(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0 && best > 0.0f) atomicMax(maxSpeedSqBits, __float_as_uint(best));
}

// --------------------------------------------------------------- liquid SDF
// One CTA per 10^3-cell block of the reference (particlelevelset.h:140-142):
// every particle whose search box reaches the block updates the block's
// cells with min(|c - p| - r) in the block's own float frame
// (particlelevelset.cpp:582-629).  Min is order-free, so the result is
// bit-identical to the reference.  Rounded square root and the subtraction
// of r are both monotone, so min over particles of fl(fl(sqrt(d2)) - r)
// equals fl(fl(sqrt(min d2)) - r): the particle loop keeps the smallest
// squared distance per cell and each cell takes one square root at the end.
// Then the solid post-process (particlelevelset.cpp:172-196).
constexpr int BW = 10;
static_assert(BW <= 15, "the SDF kernel packs block-local cell coordinates in 4 bits");

// Does the reference's count pass put particle p in block (bx,by,bz)'s list?
// (particlelevelset.cpp:477-532, velocityadvector.cpp:272-329)
__device__ __forceinline__ bool in_block_list(float px, float py, float pz, float sr, float blockdxf,
                                              double invBlock, float invBlockf, const float *blockPosF,
                                              int bx, int by, int bz) {
    int ci = exact_floor(px, invBlock, invBlockf), cj = exact_floor(py, invBlock, invBlockf),
        ck = exact_floor(pz, invBlock, invBlockf);
    // (float)((double)(float)n * (double)blockdxf), tabulated from n = -1
    float bpx = blockPosF[ci + 1], bpy = blockPosF[cj + 1], bpz = blockPosF[ck + 1];
    if (__fsub_rn(px, sr) > bpx && __fsub_rn(py, sr) > bpy && __fsub_rn(pz, sr) > bpz &&
        __fadd_rn(px, sr) < __fadd_rn(bpx, blockdxf) && __fadd_rn(py, sr) < __fadd_rn(bpy, blockdxf) &&
        __fadd_rn(pz, sr) < __fadd_rn(bpz, blockdxf)) {
        return ci == bx && cj == by && ck == bz;
    }
    int i0 = exact_floor(__fsub_rn(px, sr), invBlock, invBlockf), i1 = exact_floor(__fadd_rn(px, sr), invBlock, invBlockf);
    int j0 = exact_floor(__fsub_rn(py, sr), invBlock, invBlockf), j1 = exact_floor(__fadd_rn(py, sr), invBlock, invBlockf);
    int k0 = exact_floor(__fsub_rn(pz, sr), invBlock, invBlockf), k1 = exact_floor(__fadd_rn(pz, sr), invBlock, invBlockf);
    return bx >= i0 && bx <= i1 && by >= j0 && by <= j1 && bz >= k0 && bz <= k1;
}

// 16 warps per 10^3 block: the block's ~200 rows of candidate particles
// then take about 6 passes per warp, where 8 warps leave the blocks of a
// small scene (one wave of CTAs) bound by the latency of their atomics.
// The CTA size is a tuning knob (256, 512 or 1024 threads; default 512).
template <int SDF_TPB>
__global__ void __launch_bounds__(SDF_TPB) k_liquid_sdf(ParticleSoA p, const int *cellStart, StepConsts c,
                                                        const uint8_t *solidCC, float *phi) {
    __shared__ unsigned int smin[BW * BW * BW];   // bits of the smallest squared distance (>= 0)
    __shared__ float centre[BW];
    __shared__ float4 recs[SDF_TPB / 32][32];     // per warp: a pass's particles {lx, ly, lz, box}
    const int bx = blockIdx.x, by = blockIdx.y, bz = blockIdx.z;
    const double dx = c.dx;
    const float maxd = (float)(3.0 * dx);
    for (int q = threadIdx.x; q < BW * BW * BW; q += blockDim.x) smin[q] = 0x7f800000u;   // +inf
    if (threadIdx.x < BW) centre[threadIdx.x] = cell_centre(threadIdx.x, dx);
    __syncthreads();

    const float r = (float)c.radius;
    const float sr = __fmul_rn(2.0f, r);
    const float blockdxf = (float)(BW * dx);
    const double invBlock = 1.0 / (double)blockdxf;
    const float invBlockf = (float)invBlock;
    const float offx = c.blockPos[bx + 1], offy = c.blockPos[by + 1],
                offz = c.blockPos[bz + 1];
    Dims cells{c.I, c.J, c.K};
    int x0 = max(bx * BW - 2, 0), x1 = min(bx * BW + BW + 1, c.I - 1);
    int y0 = max(by * BW - 2, 0), y1 = min(by * BW + BW + 1, c.J - 1);
    int z0 = max(bz * BW - 2, 0), z1 = min(bz * BW + BW + 1, c.K - 1);
    int ny = y1 - y0 + 1, nrows = ny * (z1 - z0 + 1);
    // A warp takes one row of cells along x at a time and its candidate
    // particles 32 at a time.  Phase 1, a lane per particle: is it in this
    // block's list, and which of the block's cells does its box cover.  Phase
    // 2, a lane per (particle, column of the box along z): the warp's lanes
    // are spread evenly over all columns of the pass's particles (a prefix
    // sum of the column counts and a binary search), and each lane walks its
    // column.  Lanes of one step are in distinct columns of one particle, or
    // of different particles.
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    float4 *wrec = recs[warp];
    // col / n = (col * ceil(2^11 / n)) >> 11, exact for n <= BW and col < n * BW;
    // lane n holds the multiplier
    const int divLane = lane > 0 ? (2048 + lane - 1) / lane : 0;
    for (int row = warp; row < nrows; row += nwarps) {
        const int cy = y0 + row % ny, cz = z0 + row / ny;
        const int pb = cellStart[cells.idx(x0, cy, cz)];
        const int pe = cellStart[cells.idx(x1, cy, cz) + 1];
        for (int base = pb; base < pe; base += 32) {
            const int t = base + lane;
            int ncol = 0, na = 0;
            float4 rec;
            unsigned box = 0;
            if (t < pe) {
                const float px = p.px[t], py = p.py[t], pz = p.pz[t];
                if (in_block_list(px, py, pz, sr, blockdxf, invBlock, invBlockf, c.blockPosF, bx, by, bz)) {
                    const float lx = __fsub_rn(px, offx), ly = __fsub_rn(py, offy), lz = __fsub_rn(pz, offz);
                    const int a0 = max(exact_floor(__fsub_rn(lx, sr), c.invdx, c.invdxf), 0);
                    const int b0 = max(exact_floor(__fsub_rn(ly, sr), c.invdx, c.invdxf), 0);
                    const int c0 = max(exact_floor(__fsub_rn(lz, sr), c.invdx, c.invdxf), 0);
                    const int a1 = min(exact_floor(__fadd_rn(lx, sr), c.invdx, c.invdxf), BW - 1);
                    const int b1 = min(exact_floor(__fadd_rn(ly, sr), c.invdx, c.invdxf), BW - 1);
                    const int c1 = min(exact_floor(__fadd_rn(lz, sr), c.invdx, c.invdxf), BW - 1);
                    if (a1 >= a0 && b1 >= b0 && c1 >= c0) {
                        na = a1 - a0 + 1;
                        ncol = na * (b1 - b0 + 1);
                        box = (unsigned)a0 | (unsigned)na << 4 | (unsigned)b0 << 8 | (unsigned)c0 << 12 |
                              (unsigned)c1 << 16;
                        rec = make_float4(lx, ly, lz, 0.0f);
                    }
                }
            }
            const unsigned div = (unsigned)__shfl_sync(0xffffffffu, divLane, na);
            if (ncol > 0) {
                rec.w = __uint_as_float(box | div << 20);
                wrec[lane] = rec;
            }
            int incl = ncol;   // inclusive prefix sum of the column counts over the lanes
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            __syncwarp();
            for (int first = 0; first < total; first += 32) {
                const int item = first + lane;
                int L = 0;   // the smallest lane whose inclusive sum exceeds item
#pragma unroll
                for (int step = 16; step > 0; step >>= 1)
                    if (__shfl_sync(0xffffffffu, incl, L + step - 1) <= item) L += step;
                const int startL = __shfl_sync(0xffffffffu, incl, L) - __shfl_sync(0xffffffffu, ncol, L);
                if (item < total) {
                    const float4 pr = wrec[L];
                    const unsigned w = __float_as_uint(pr.w);
                    const int a0 = w & 15, na = (w >> 4) & 15, b0 = (w >> 8) & 15;
                    const int c0 = (w >> 12) & 15, c1 = (w >> 16) & 15;
                    const int col = item - startL;
                    const int bq = (col * (int)(w >> 20)) >> 11;   // col / na
                    const int aa = a0 + col - bq * na, bb = b0 + bq;
                    const float ddx = __fsub_rn(centre[aa], pr.x);
                    const float dy = __fsub_rn(centre[bb], pr.y);
                    const float dxy = __fadd_rn(__fmul_rn(ddx, ddx), __fmul_rn(dy, dy));
                    unsigned int *dst = &smin[aa + BW * (bb + BW * c0)];
                    for (int cc = c0; cc <= c1; cc++, dst += BW * BW) {
                        const float dz = __fsub_rn(centre[cc], pr.z);
                        atomicMin(dst, __float_as_uint(__fadd_rn(dxy, __fmul_rn(dz, dz))));
                    }
                }
            }
            __syncwarp();
        }
    }
    __syncthreads();
    const float eps = (float)(0.005 * dx);
    const double half = 0.5 * dx;
    const float neg = (float)(-0.5f * dx);
    for (int q = threadIdx.x; q < BW * BW * BW; q += blockDim.x) {
        int a = q % BW, b = (q / BW) % BW, cz = q / (BW * BW);
        int gi = bx * BW + a, gj = by * BW + b, gk = bz * BW + cz;
        if (!cells.in(gi, gj, gk)) continue;
        long long ci = cells.idx(gi, gj, gk);
        const unsigned int m = smin[q];
        float val = m == 0x7f800000u ? maxd : fminf(maxd, __fsub_rn(__fsqrt_rn(__uint_as_float(m)), r));
        if ((double)val < half && solidCC[ci]) val = neg;
        if (fabsf(val) < eps) val = val > 0 ? eps : -eps;
        phi[ci] = val;
    }
}

// ---------------------------------------------------------------------- P2G
// Gather form of VelocityAdvector (velocityadvector.cpp:38-459): one thread
// per face; candidate particles come from the 18 cells that can hold a
// particle within r of the face; each particle's weight is evaluated in the
// reference's 10^3-block frame.  Sums run in a fixed (cell, id) order, so
// the result is deterministic (no float atomics).
__global__ void __launch_bounds__(TPB) k_p2g(ParticleSoA p, const int *cellStart, StepConsts c, int dir,
                                             float *G, uint8_t *valid) {
    const int ni = c.I + (dir == 0), nj = c.J + (dir == 1), nk = c.K + (dir == 2);
    long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= (long long)ni * nj * nk) return;
    int fi, fj, fk;
    unflatten(f, ni, nj, fi, fj, fk);
    const double dx = c.dx;
    const float r = (float)c.radius;
    const float rsq = __fmul_rn(r, r);
    // same expression trees as the reference's coefficient set-up
    const float coef1 = __fmul_rn(4.0f / 9.0f, __fdiv_rn(1.0f, __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(r, r), r), r), r), r)));
    const float coef2 = __fmul_rn(17.0f / 9.0f, __fdiv_rn(1.0f, __fmul_rn(__fmul_rn(__fmul_rn(r, r), r), r)));
    const float coef3 = __fmul_rn(22.0f / 9.0f, __fdiv_rn(1.0f, __fmul_rn(r, r)));
    const float halfdx = (float)(0.5 * dx);
    const float ox = dir == 0 ? 0.0f : halfdx, oy = dir == 1 ? 0.0f : halfdx, oz = dir == 2 ? 0.0f : halfdx;
    const int bx = fi / BW, by = fj / BW, bz = fk / BW;
    const float offx = c.blockPos[bx + 1], offy = c.blockPos[by + 1],
                offz = c.blockPos[bz + 1];
    const int la = fi - bx * BW, lb = fj - by * BW, lc = fk - bz * BW;
    const float gx = c.nodePos[la], gy = c.nodePos[lb], gz = c.nodePos[lc];
    // candidate cells of the cell grid
    int cx0 = dir == 0 ? fi - 1 : fi - 1, cx1 = dir == 0 ? fi : fi + 1;
    int cy0 = fj - 1, cy1 = dir == 1 ? fj : fj + 1;
    int cz0 = fk - 1, cz1 = dir == 2 ? fk : fk + 1;
    cx0 = max(cx0, 0); cy0 = max(cy0, 0); cz0 = max(cz0, 0);
    cx1 = min(cx1, c.I - 1); cy1 = min(cy1, c.J - 1); cz1 = min(cz1, c.K - 1);
    Dims cells{c.I, c.J, c.K};
    float sc = 0.0f, wt = 0.0f;
    for (int cz = cz0; cz <= cz1; cz++)
        for (int cy = cy0; cy <= cy1; cy++) {
            int pb = cellStart[cells.idx(cx0, cy, cz)], pe = cellStart[cells.idx(cx1, cy, cz) + 1];
            for (int t = pb; t < pe; t++) {
                float px = __fsub_rn(p.px[t], ox), py = __fsub_rn(p.py[t], oy), pz = __fsub_rn(p.pz[t], oz);
                float lx = __fsub_rn(px, offx), ly = __fsub_rn(py, offy), lz = __fsub_rn(pz, offz);
                float ddx = __fsub_rn(gx, lx), ddy = __fsub_rn(gy, ly), ddz = __fsub_rn(gz, lz);
                float d2 = __fadd_rn(__fadd_rn(__fmul_rn(ddx, ddx), __fmul_rn(ddy, ddy)), __fmul_rn(ddz, ddz));
                if (!(d2 < rsq)) continue;
                // The reference also requires the face to lie in the particle's
                // local box and the particle to be in the block's list, both
                // taken with the support radius sr = r + 1e-6.  A particle
                // within r of the face meets both: every coordinate of the face
                // is within r of the particle, and the 1e-6 margin is far above
                // the rounding of these float expressions (ulp(1) ~ 1.2e-7).
                float vel = dir == 0 ? p.vx[t] : dir == 1 ? p.vy[t] : p.vz[t];
                float w3 = __fmul_rn(__fmul_rn(__fmul_rn(coef1, d2), d2), d2);
                float w2 = __fmul_rn(__fmul_rn(coef2, d2), d2);
                float w1 = __fmul_rn(coef3, d2);
                float wgt = __fsub_rn(__fadd_rn(__fsub_rn(1.0f, w3), w2), w1);
                sc = __fadd_rn(sc, __fmul_rn(wgt, vel));
                wt = __fadd_rn(wt, wgt);
            }
        }
    const float eps = 1e-6f;
    bool ok = wt > eps;
    if (ok) sc = __fdiv_rn(sc, wt);
    G[f] = sc;
    valid[f] = ok ? 1 : 0;
}

// ------------------------------------------------------------ extrapolation
// Layered BFS of GridUtils::extrapolateGrid (gridutils.cpp:32-228) done in
// place, one launch per layer.  Status: 0 = valid input, l+1 = filled by
// layer l, 254 = grid border (fixed, counts as known), 255 = unknown.
constexpr uint8_t ST_BORDER = 254, ST_UNKNOWN = 255;

__global__ void k_extrap_init(StepConsts c, const uint8_t *vu, const uint8_t *vv, const uint8_t *vw,
                              uint8_t *status) {
    long long nu = (long long)(c.I + 1) * c.J * c.K, nv = (long long)c.I * (c.J + 1) * c.K;
    long long nw = (long long)c.I * c.J * (c.K + 1);
    long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nu + nv + nw) return;
    int dir = f < nu ? 0 : (f < nu + nv ? 1 : 2);
    long long l = dir == 0 ? f : (dir == 1 ? f - nu : f - nu - nv);
    const uint8_t *valid = dir == 0 ? vu : (dir == 1 ? vv : vw);
    int ni = c.I + (dir == 0), nj = c.J + (dir == 1), nk = c.K + (dir == 2);
    int i, j, k;
    unflatten(l, ni, nj, i, j, k);
    uint8_t s;
    if (i == 0 || j == 0 || k == 0 || i == ni - 1 || j == nj - 1 || k == nk - 1) s = ST_BORDER;
    else s = valid[l] ? 0 : ST_UNKNOWN;
    status[f] = s;
}

__global__ void k_extrap_layer(StepConsts c, float *u, float *v, float *w, uint8_t *status, int layer) {
    long long nu = (long long)(c.I + 1) * c.J * c.K, nv = (long long)c.I * (c.J + 1) * c.K;
    long long nw = (long long)c.I * c.J * (c.K + 1);
    long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nu + nv + nw) return;
    if (status[f] != ST_UNKNOWN) return;
    int dir = f < nu ? 0 : (f < nu + nv ? 1 : 2);
    long long base = dir == 0 ? 0 : (dir == 1 ? nu : nu + nv);
    long long l = f - base;
    float *G = dir == 0 ? u : (dir == 1 ? v : w);
    int ni = c.I + (dir == 0), nj = c.J + (dir == 1);
    long long sx = 1, sy = ni, sz = (long long)ni * nj;
    // unknown cells are never on the border, so all six neighbours exist
    const long long nb[6] = {l + sx, l - sx, l + sy, l - sy, l + sz, l - sz};
    bool frontier = false;
#pragma unroll
    for (int q = 0; q < 6; q++) frontier |= status[base + nb[q]] == (uint8_t)layer;
    if (!frontier) return;
    float sum = 0.0f;
    int count = 0;
#pragma unroll
    for (int q = 0; q < 6; q++) {
        uint8_t s = status[base + nb[q]];
        if (s == ST_BORDER || s <= (uint8_t)layer) {
            sum = __fadd_rn(sum, G[nb[q]]);
            count++;
        }
    }
    G[l] = __fdiv_rn(sum, (float)count);
    status[f] = (uint8_t)(layer + 1);
}

// -------------------------------------------------- save + body force, constrain
// `ex` (optional, one byte per face over u, v, w): faces an inflow source
// constrains, which the body force skips (fluidsimulation.cpp:3450-3489).
__global__ void k_save_force(long long nu, long long nv, long long nw, float *u, float *v, float *w, float *su,
                             float *sv, float *sw, float fx, float fy, float fz, int ax, int ay, int az,
                             const uint8_t *ex) {
    long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool skip = ex && f < nu + nv + nw && ex[f];
    if (f < nu) {
        float x = u[f]; su[f] = x; if (ax && !skip) u[f] = __fadd_rn(x, fx);
    } else if (f < nu + nv) {
        long long l = f - nu; float x = v[l]; sv[l] = x; if (ay && !skip) v[l] = __fadd_rn(x, fy);
    } else if (f < nu + nv + nw) {
        long long l = f - nu - nv; float x = w[l]; sw[l] = x; if (az && !skip) w[l] = __fadd_rn(x, fz);
    }
}

// Faces with zero fluid weight take the solid velocity, which is zero for
// static solids; partly solid faces blend it with their own velocity by the
// mean friction of the solid objects closest to their four corners
// (src/engine/fluidsimulation.cpp:3785-3846, 3884-3950).  The domain walls
// have no friction: without friction arrays those faces stay as they are.
__global__ void k_constrain(long long nu, long long nv, long long nw, float *u, float *v, float *w, float *su,
                            float *sv, float *sw, const float *wu, const float *wv, const float *ww, const float *fu,
                            const float *fv, const float *fw) {
    long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    float *G, *S;
    const float *W, *F;
    long long l;
    if (f < nu) { G = u; S = su; W = wu; F = fu; l = f; }
    else if (f < nu + nv) { G = v; S = sv; W = wv; F = fv; l = f - nu; }
    else if (f < nu + nv + nw) { G = w; S = sw; W = ww; F = fw; l = f - nu - nv; }
    else return;
    const float wt = W[l];
    if (wt == 0.0f) {   // inside the solid: the solid's velocity (zero for static solids)
        G[l] = 0.0f;
        if (S) S[l] = 0.0f;
    } else if (wt < 1.0f && F) {   // part solid: f usolid + (1 - f) u, usolid = 0
        const float fr = F[l], keep = __fsub_rn(1.0f, fr), us = __fmul_rn(fr, 0.0f);
        G[l] = __fadd_rn(us, __fmul_rn(keep, G[l]));
        if (S) S[l] = __fadd_rn(us, __fmul_rn(keep, S[l]));
    }
}

// ---------------------------------------------------------- particle update
// Trilinear weights of Interpolation::trilinearInterpolate (interpolation.cpp:
// 61-70) with vertex order {000,100,010,001,101,011,110,111}, in FP32.
__device__ __forceinline__ float trilerp_f(const float q[8], float x, float y, float z) {
    float x1 = 1.0f - x, y1 = 1.0f - y, z1 = 1.0f - z;
    float r = q[0] * (x1 * y1 * z1);
    r = __fmaf_rn(q[1], x * y1 * z1, r);
    r = __fmaf_rn(q[2], x1 * y * z1, r);
    r = __fmaf_rn(q[3], x1 * y1 * z, r);
    r = __fmaf_rn(q[4], x * y1 * z, r);
    r = __fmaf_rn(q[5], x1 * y * z, r);
    r = __fmaf_rn(q[6], x * y * z1, r);
    r = __fmaf_rn(q[7], x * y * z, r);
    return r;
}

__device__ __forceinline__ float grid_at(const float *G, int ni, int nj, int nk, int a, int b, int cc) {
    bool in = a >= 0 && b >= 0 && cc >= 0 && a < ni && b < nj && cc < nk;
    return in ? __ldg(&G[(long long)a + (long long)ni * ((long long)b + (long long)nj * cc)]) : 0.0f;
}

// MAC velocity component at a point, as MACVelocityField::_interpolateLinearU/V/W
// (macvelocityfield.cpp:519-613) but in FP32.  The cell coordinate is
// x*(1/dx) - 1/2 in one fused step, which is exact for power-of-two dx and
// within half an ulp otherwise; the reference evaluates the same in FP64.
__device__ __forceinline__ float interp_face(const float *G, int ni, int nj, int nk, int dir, float x, float y,
                                             float z, float invdxf) {
    float fx = dir == 0 ? __fmul_rn(x, invdxf) : __fmaf_rn(x, invdxf, -0.5f);
    float fy = dir == 1 ? __fmul_rn(y, invdxf) : __fmaf_rn(y, invdxf, -0.5f);
    float fz = dir == 2 ? __fmul_rn(z, invdxf) : __fmaf_rn(z, invdxf, -0.5f);
    float gi = floorf(fx), gj = floorf(fy), gk = floorf(fz);
    int i = (int)gi, j = (int)gj, k = (int)gk;
    float q[8] = {grid_at(G, ni, nj, nk, i, j, k),         grid_at(G, ni, nj, nk, i + 1, j, k),
                  grid_at(G, ni, nj, nk, i, j + 1, k),     grid_at(G, ni, nj, nk, i, j, k + 1),
                  grid_at(G, ni, nj, nk, i + 1, j, k + 1), grid_at(G, ni, nj, nk, i, j + 1, k + 1),
                  grid_at(G, ni, nj, nk, i + 1, j + 1, k), grid_at(G, ni, nj, nk, i + 1, j + 1, k + 1)};
    return trilerp_f(q, fx - gi, fy - gj, fz - gk);
}

// isPositionInGrid (grid3d.h:133-135): x >= 0 && x < I dx, with the upper
// bound pre-rounded so the float compare equals the reference's FP64 one.
__device__ __forceinline__ bool in_grid(const StepConsts &c, F3 p) {
    return p.x >= 0.0f && p.y >= 0.0f && p.z >= 0.0f && p.x <= c.gxmax && p.y <= c.gymax && p.z <= c.gzmax;
}

__device__ F3 eval_vel(const StepConsts &c, const float *u, const float *v, const float *w, F3 p) {
    if (!in_grid(c, p)) return f3(0.0f, 0.0f, 0.0f);
    return f3(interp_face(u, c.I + 1, c.J, c.K, 0, p.x, p.y, p.z, c.invdxf),
              interp_face(v, c.I, c.J + 1, c.K, 1, p.x, p.y, p.z, c.invdxf),
              interp_face(w, c.I, c.J, c.K + 1, 2, p.x, p.y, p.z, c.invdxf));
}

// Nodal solid SDF at a point (Interpolation::trilinearInterpolate(vec3, dx,
// grid), interpolation.cpp:72-113).  FP32 weights; when the value is within
// rounding of zero the sign is settled by the reference's FP64 evaluation.
__device__ float solid_at(const StepConsts &c, const float *S, F3 p) {
    int i = exact_floor(p.x, c.invdx, c.invdxf), j = exact_floor(p.y, c.invdx, c.invdxf),
        k = exact_floor(p.z, c.invdx, c.invdxf);
    float dxl = __fsub_rn(p.x, c.nodePos[max(i, 0)]), dyl = __fsub_rn(p.y, c.nodePos[max(j, 0)]),
          dzl = __fsub_rn(p.z, c.nodePos[max(k, 0)]);
    int ni = c.I + 1, nj = c.J + 1, nk = c.K + 1;
    float q[8] = {grid_at(S, ni, nj, nk, i, j, k),         grid_at(S, ni, nj, nk, i + 1, j, k),
                  grid_at(S, ni, nj, nk, i, j + 1, k),     grid_at(S, ni, nj, nk, i, j, k + 1),
                  grid_at(S, ni, nj, nk, i + 1, j, k + 1), grid_at(S, ni, nj, nk, i, j + 1, k + 1),
                  grid_at(S, ni, nj, nk, i + 1, j + 1, k), grid_at(S, ni, nj, nk, i + 1, j + 1, k + 1)};
    float v = trilerp_f(q, dxl * c.invdxf, dyl * c.invdxf, dzl * c.invdxf);
    float mag = 0.0f;
#pragma unroll
    for (int t = 0; t < 8; t++) mag += fabsf(q[t]);
    if (fabsf(v) > 1e-6f * mag) return v;
    double qd[8];
#pragma unroll
    for (int t = 0; t < 8; t++) qd[t] = q[t];
    double ix = (double)dxl * c.invdx, iy = (double)dyl * c.invdx, iz = (double)dzl * c.invdx;
    return (float)(qd[0] * (1 - ix) * (1 - iy) * (1 - iz) + qd[1] * ix * (1 - iy) * (1 - iz) +
                   qd[2] * (1 - ix) * iy * (1 - iz) + qd[3] * (1 - ix) * (1 - iy) * iz + qd[4] * ix * (1 - iy) * iz +
                   qd[5] * (1 - ix) * iy * iz + qd[6] * ix * iy * (1 - iz) + qd[7] * ix * iy * iz);
}

// Interpolation::trilinearInterpolateGradient (interpolation.cpp:197-258), FP32
__device__ F3 solid_grad(const StepConsts &c, const float *S, F3 p) {
    int i = exact_floor(p.x, c.invdx, c.invdxf), j = exact_floor(p.y, c.invdx, c.invdxf),
        k = exact_floor(p.z, c.invdx, c.invdxf);
    float ix = __fsub_rn(p.x, c.nodePos[max(i, 0)]) * c.invdxf;
    float iy = __fsub_rn(p.y, c.nodePos[max(j, 0)]) * c.invdxf;
    float iz = __fsub_rn(p.z, c.nodePos[max(k, 0)]) * c.invdxf;
    int ni = c.I + 1, nj = c.J + 1, nk = c.K + 1;
    float v000 = grid_at(S, ni, nj, nk, i, j, k), v100 = grid_at(S, ni, nj, nk, i + 1, j, k);
    float v010 = grid_at(S, ni, nj, nk, i, j + 1, k), v001 = grid_at(S, ni, nj, nk, i, j, k + 1);
    float v101 = grid_at(S, ni, nj, nk, i + 1, j, k + 1), v011 = grid_at(S, ni, nj, nk, i, j + 1, k + 1);
    float v110 = grid_at(S, ni, nj, nk, i + 1, j + 1, k), v111 = grid_at(S, ni, nj, nk, i + 1, j + 1, k + 1);
    auto bil = [](float a, float b, float cc, float d, float x, float y) {
        float l1 = (1 - x) * a + x * b;
        float l2 = (1 - x) * cc + x * d;
        return (1 - y) * l1 + y * l2;
    };
    float gx = bil(v100 - v000, v110 - v010, v101 - v001, v111 - v011, iy, iz);
    float gy = bil(v010 - v000, v110 - v100, v011 - v001, v111 - v101, ix, iz);
    float gz = bil(v001 - v000, v101 - v100, v011 - v010, v111 - v110, ix, iy);
    return f3(gx, gy, gz);
}

__device__ __forceinline__ bool box_inside(const StepConsts &c, F3 p) {
    return p.x >= c.bposx && p.y >= c.bposy && p.z >= c.bposz && (double)p.x < (double)c.bposx + c.bw &&
           (double)p.y < (double)c.bposy + c.bh && (double)p.z < (double)c.bposz + c.bd;
}
// AABB::getNearestPointInsideAABB (aabb.cpp:497-518), eps 1e-6
__device__ __forceinline__ F3 box_nearest(const StepConsts &c, F3 p) {
    if (box_inside(c, p)) return p;
    float mxx = __fadd_rn(c.bposx, (float)c.bw);
    float mxy = __fadd_rn(c.bposy, (float)c.bh);
    float mxz = __fadd_rn(c.bposz, (float)c.bd);
    p.x = fmaxf(p.x, c.bposx); p.y = fmaxf(p.y, c.bposy); p.z = fmaxf(p.z, c.bposz);
    p.x = (float)fmin((double)p.x, (double)mxx - 1e-6);
    p.y = (float)fmin((double)p.y, (double)mxy - 1e-6);
    p.z = (float)fmin((double)p.z, (double)mxz - 1e-6);
    return p;
}

__device__ __forceinline__ bool near_solid(const StepConsts &c, const uint8_t *ns, F3 p) {
    int i = exact_floor(p.x, c.invNearCell, c.invNearCellf), j = exact_floor(p.y, c.invNearCell, c.invNearCellf),
        k = exact_floor(p.z, c.invNearCell, c.invNearCellf);
    if (i < 0 || j < 0 || k < 0 || i >= c.nsi || j >= c.nsj || k >= c.nsk) return false;
    return ns[(long long)i + (long long)c.nsi * ((long long)j + (long long)c.nsj * k)] != 0;
}

// FluidSimulation::_resolveCollision (src/engine/fluidsimulation.cpp:4221-4296)
__device__ F3 resolve_collision(const StepConsts &c, const float *S, const uint8_t *ns, F3 oldp, F3 newp) {
    int gi = exact_floor(newp.x, c.invdx, c.invdxf), gj = exact_floor(newp.y, c.invdx, c.invdxf),
        gk = exact_floor(newp.z, c.invdx, c.invdxf);
    if (!(gi >= 0 && gj >= 0 && gk >= 0 && gi < c.I && gj < c.J && gk < c.K)) newp = box_nearest(c, newp);
    if (!near_solid(c, ns, oldp) && !near_solid(c, ns, newp)) return newp;
    const float eps = 1e-6f;
    const float stepDist = __fmul_rn(0.5f, (float)c.dx);
    float travel = len3(sub(newp, oldp));
    if (travel < eps) return newp;
    int nsteps = (int)ceilf(__fdiv_rn(travel, stepDist));
    F3 dir = normalize3(sub(newp, oldp));
    F3 last = oldp, cur = oldp;
    bool found = false;
    float cphi = 0.0f;
    for (int s = 0; s < nsteps; s++) {
        if (s == nsteps - 1) cur = newp;
        else cur = add(oldp, mul(__fmul_rn((float)(s + 1), stepDist), dir));
        float ph = solid_at(c, S, cur);
        if (ph < 0.0f || !box_inside(c, cur)) { cphi = ph; found = true; break; }
        last = cur;
    }
    if (!found) return newp;
    F3 res;
    const float maxDist = (float)(c.cfl * c.dx);
    F3 g = solid_grad(c, S, cur);
    if (len3(g) > eps) {
        g = normalize3(g);
        res = sub(cur, mul((float)((double)cphi - (double)0.1f * c.dx), g));
        float rphi = solid_at(c, S, res);
        float rd = len3(sub(res, cur));
        if (rphi < 0 || rd > maxDist) res = last;
    } else {
        res = last;
    }
    if (!box_inside(c, res)) {
        F3 orig = res;
        res = box_nearest(c, res);
        float rphi = solid_at(c, S, res);
        float rd = len3(sub(res, orig));
        if (rphi < 0.0f || rd > maxDist) res = last;
    }
    return res;
}

// Fused particle update: PIC/FLIP velocity (fluidsimulation.cpp:4082-4092),
// Ralston RK3 (4191-4198), collision (4221-4296), then the removal tests and
// the new cell key for the next binning.
__global__ void __launch_bounds__(TPB) k_advect(ParticleSoA p, int n, StepConsts c, const float *u, const float *v,
                                                const float *w, const float *su, const float *sv, const float *sw,
                                                const float *S, const uint8_t *ns, float picRatio, float flipRatio,
                                                double dt, unsigned int *keys, unsigned int *hist, double speedStep,
                                                const InflowConstraint ic) {
    __shared__ unsigned int shist[8];
    if (threadIdx.x < 8) shist[threadIdx.x] = 0;
    __syncthreads();
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        F3 p0 = f3(p.px[t], p.py[t], p.pz[t]);
        F3 v0 = f3(p.vx[t], p.vy[t], p.vz[t]);
        F3 vpic = eval_vel(c, u, v, w, p0);
        F3 vold = eval_vel(c, su, sv, sw, p0);
        F3 vflip = sub(add(v0, vpic), vold);
        F3 vn = add(mul(picRatio, vpic), mul(flipRatio, vflip));
        if (ic.count > 0) {
            // _constrainMarkerParticleVelocities (fluidsimulation.cpp:4109-4170):
            // a particle in a cell of the source where the source's level set,
            // read at the particle's position in the level set's own frame (the
            // reference passes the position without the level set's offset), is
            // not positive takes the source's velocity; later sources win
            const int ci = exact_floor(p0.x, c.invdx, c.invdxf), cj = exact_floor(p0.y, c.invdx, c.invdxf),
                      ck = exact_floor(p0.z, c.invdx, c.invdxf);
            const Dims d{c.I, c.J, c.K};
            const unsigned bits = d.in(ci, cj, ck) ? ic.cellBits[d.idx(ci, cj, ck)] : 0u;
            for (int q = 0; q < ic.count; q++)
                if ((bits >> q & 1u) && !(source_phi(ic.g[q], p0.x, p0.y, p0.z) > 0.0f))
                    vn = f3(ic.vx[q], ic.vy[q], ic.vz[q]);
        }
        F3 k1 = vpic;
        F3 k2 = eval_vel(c, u, v, w, add(p0, mul((float)(0.5 * dt), k1)));
        F3 k3 = eval_vel(c, u, v, w, add(p0, mul((float)(0.75 * dt), k2)));
        F3 sum = add(add(mul(2.0f, k1), mul(3.0f, k2)), mul(4.0f, k3));
        F3 p1 = add(p0, mul((float)(dt / 9.0f), sum));
        p1 = resolve_collision(c, S, ns, p0, p1);
        p.px[t] = p1.x; p.py[t] = p1.y; p.pz[t] = p1.z;
        p.vx[t] = vn.x; p.vy[t] = vn.y; p.vz[t] = vn.z;
        float speed = len3(vn);
        // floor(speed / step) as the reference's FP64 division gives it
        float qf = __fmul_rn(speed, (float)(1.0 / speedStep));
        float fl = floorf(qf);
        int bin = (qf - fl > 1e-3f && qf - fl < 1.0f - 1e-3f) ? (int)fminf(fl, 5.0f)
                                                               : (int)fmin(floor((double)speed / speedStep), 5.0);
        if (speed != speed) bin = 5;
        atomicAdd(&shist[bin], 1u);
        unsigned int key;
        if (solid_at(c, S, p1) < 0.0f) {
            key = KEY_SOLID;
        } else {
            int i = exact_floor(p1.x, c.invdx, c.invdxf), j = exact_floor(p1.y, c.invdx, c.invdxf),
                k = exact_floor(p1.z, c.invdx, c.invdxf);
            Dims d{c.I, c.J, c.K};
            key = d.in(i, j, k) ? (unsigned int)d.idx(i, j, k) : KEY_SOLID;
        }
        keys[t] = key;
    }
    __syncthreads();
    if (threadIdx.x < 6 && shist[threadIdx.x]) atomicAdd(&hist[threadIdx.x], shist[threadIdx.x]);
}

// _getMarkerParticleSpeedLimit (fluidsimulation.cpp:4298-4322), one thread
__global__ void k_speed_limit(const unsigned int *hist, int n, int bins, double step, double maxPct, int maxAbs,
                              float *maxSpeedSq) {
    int maxRemoval = (int)fmin((double)(int)((double)n * maxPct), (double)maxAbs);
    double maxspeed = bins * step;
    int cur = 0;
    for (int i = bins - 1; i > 0; i--) {
        if (cur + (int)hist[i] > maxRemoval) break;
        cur += (int)hist[i];
        maxspeed = i * step;
    }
    float ms = (float)maxspeed;
    *maxSpeedSq = __fmul_rn(ms, ms);
}

__global__ void k_mark_fast(ParticleSoA p, int n, const float *maxSpeedSq, unsigned int *keys) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    unsigned int k = keys[t];
    if (k & KEY_SOLID) return;
    F3 v = f3(p.vx[t], p.vy[t], p.vz[t]);
    if (dot3(v, v) > *maxSpeedSq) keys[t] = k | KEY_FAST;
}

}  // namespace

// ------------------------------------------------------------------ launchers
void launch_keys_from_positions(const ParticleSoA &p, int n, const StepConsts &c, unsigned int *keys, cudaStream_t s) {
    if (n > 0) { FLIP_COUNT(1); k_keys<<<div_up(n, TPB), TPB, 0, s>>>(p, n, c, keys); }
}
void launch_bin_count(const unsigned int *keys, int n, int *cellCount, cudaStream_t s) {
    if (n > 0) { FLIP_COUNT(1); k_bin_count<<<div_up(n, TPB), TPB, 0, s>>>(keys, n, cellCount); }
}
int scan_scratch_ints(int ncells) { return (int)div_up(ncells + 1, SCAN_TILE) + 2; }
void launch_scan_cells(const int *count, int ncells, int *start, int *scratch, int *total, cudaStream_t s) {
    int ntiles = (int)div_up(ncells, SCAN_TILE);
    { FLIP_COUNT(1); k_scan_tiles<<<ntiles, SCAN_T, 0, s>>>(count, ncells, start, scratch); }
    { FLIP_COUNT(1); k_scan_sums<<<1, SCAN_T, 0, s>>>(scratch, ntiles, total); }
    { FLIP_COUNT(1); k_scan_add<<<div_up(ncells + 1, TPB), TPB, 0, s>>>(start, ncells, scratch, total); }
}
void launch_bin_scatter(const unsigned int *keys, int n, const int *cellStart, int *cursor, int *slots, cudaStream_t s) {
    if (n > 0) { FLIP_COUNT(1); k_bin_scatter<<<div_up(n, TPB), TPB, 0, s>>>(keys, n, cellStart, cursor, slots); }
}
void launch_cell_sort_select(const int *cellStart, int ncells, int *slots, const unsigned int *ids,
                             const unsigned int *keys, int maxPerCell, int *survivorCount, cudaStream_t s) {
    { FLIP_COUNT(1); k_cell_sort_select<<<div_up(ncells, TPB), TPB, 0, s>>>(cellStart, ncells, slots, ids, keys, maxPerCell, survivorCount); }
}
void launch_gather_particles(const ParticleSoA &src, ParticleSoA dst, const int *cellStart, const int *slots,
                             const int *newStart, int ncells, unsigned int *maxSpeedSqBits, cudaStream_t s) {
    { FLIP_COUNT(1); k_gather<<<div_up(ncells, TPB), TPB, 0, s>>>(src, dst, cellStart, slots, newStart, ncells, maxSpeedSqBits); }
}
void launch_liquid_sdf(const ParticleSoA &p, const int *cellStart, const StepConsts &c, const uint8_t *solidCC,
                       float *phi, int threads, cudaStream_t s) {
    dim3 grid(div_up(c.I, BW), div_up(c.J, BW), div_up(c.K, BW));
    FLIP_COUNT(1);
    if (threads == 256) k_liquid_sdf<256><<<grid, 256, 0, s>>>(p, cellStart, c, solidCC, phi);
    else if (threads == 1024) k_liquid_sdf<1024><<<grid, 1024, 0, s>>>(p, cellStart, c, solidCC, phi);
    else k_liquid_sdf<512><<<grid, 512, 0, s>>>(p, cellStart, c, solidCC, phi);
}
void launch_p2g(const ParticleSoA &p, const int *cellStart, const StepConsts &c, float *u, float *v, float *w,
                uint8_t *vu, uint8_t *vv, uint8_t *vw, cudaStream_t s) {
    long long nu = (long long)(c.I + 1) * c.J * c.K, nv = (long long)c.I * (c.J + 1) * c.K,
              nw = (long long)c.I * c.J * (c.K + 1);
    { FLIP_COUNT(1); k_p2g<<<div_up(nu, TPB), TPB, 0, s>>>(p, cellStart, c, 0, u, vu); }
    { FLIP_COUNT(1); k_p2g<<<div_up(nv, TPB), TPB, 0, s>>>(p, cellStart, c, 1, v, vv); }
    { FLIP_COUNT(1); k_p2g<<<div_up(nw, TPB), TPB, 0, s>>>(p, cellStart, c, 2, w, vw); }
}
void launch_extrapolate(const StepConsts &c, float *u, float *v, float *w, const uint8_t *vu, const uint8_t *vv,
                        const uint8_t *vw, uint8_t *status, int layers, cudaStream_t s) {
    long long tot = (long long)(c.I + 1) * c.J * c.K + (long long)c.I * (c.J + 1) * c.K +
                    (long long)c.I * c.J * (c.K + 1);
    { FLIP_COUNT(1); k_extrap_init<<<div_up(tot, TPB), TPB, 0, s>>>(c, vu, vv, vw, status); }
    for (int l = 0; l < layers; l++) { FLIP_COUNT(1); k_extrap_layer<<<div_up(tot, TPB), TPB, 0, s>>>(c, u, v, w, status, l); }
}
void launch_save_and_force(const StepConsts &c, float *u, float *v, float *w, float *su, float *sv, float *sw,
                           float fx, float fy, float fz, bool ax, bool ay, bool az, const uint8_t *ex,
                           cudaStream_t s) {
    long long nu = (long long)(c.I + 1) * c.J * c.K, nv = (long long)c.I * (c.J + 1) * c.K,
              nw = (long long)c.I * c.J * (c.K + 1);
    { FLIP_COUNT(1); k_save_force<<<div_up(nu + nv + nw, TPB), TPB, 0, s>>>(nu, nv, nw, u, v, w, su, sv, sw, fx, fy, fz, ax, ay, az, ex); }
}
void launch_constrain(const StepConsts &c, float *u, float *v, float *w, float *su, float *sv, float *sw,
                      const float *wu, const float *wv, const float *ww, const float *fu, const float *fv,
                      const float *fw, cudaStream_t s) {
    long long nu = (long long)(c.I + 1) * c.J * c.K, nv = (long long)c.I * (c.J + 1) * c.K,
              nw = (long long)c.I * c.J * (c.K + 1);
    { FLIP_COUNT(1); k_constrain<<<div_up(nu + nv + nw, TPB), TPB, 0, s>>>(nu, nv, nw, u, v, w, su, sv, sw, wu, wv, ww, fu, fv, fw); }
}
void launch_advect(ParticleSoA p, int n, const StepConsts &c, const float *u, const float *v, const float *w,
                   const float *su, const float *sv, const float *sw, const float *solidPhi,
                   const uint8_t *nearSolid, float picRatio, float flipRatio, double dt, unsigned int *keys,
                   unsigned int *speedHist, double speedStep, const InflowConstraint &ic, cudaStream_t s) {
    if (n <= 0) return;
    FLIP_COUNT(1);
    k_advect<<<div_up(n, TPB), TPB, 0, s>>>(p, n, c, u, v, w, su, sv, sw, solidPhi, nearSolid, picRatio,
                                            flipRatio, dt, keys, speedHist, speedStep, ic);
}
void launch_speed_limit(const unsigned int *hist, int n, int bins, double speedStep, double maxPct, int maxAbs,
                        float *maxSpeedSq, cudaStream_t s) {
    { FLIP_COUNT(1); k_speed_limit<<<1, 1, 0, s>>>(hist, n, bins, speedStep, maxPct, maxAbs, maxSpeedSq); }
}
void launch_mark_fast(const ParticleSoA &p, int n, const float *maxSpeedSq, unsigned int *keys, cudaStream_t s) {
    if (n > 0) { FLIP_COUNT(1); k_mark_fast<<<div_up(n, TPB), TPB, 0, s>>>(p, n, maxSpeedSq, keys); }
}

}  // namespace flip
