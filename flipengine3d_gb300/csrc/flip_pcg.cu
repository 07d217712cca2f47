// Variational pressure projection for GB300 (sm_103a).
//
// The system is the reference's (pressuresolver.cpp:580-808): a 7-point
// matrix over the interior cells with phi < 0, ghost-fluid diagonal terms at
// air neighbours, face weights from the solid level set.  Its rows are built
// in FP64 exactly as the reference builds them and kept as {diag, +x, +y, +z}.
// Preconditioner: the reference's MIC(0) (pcgsolver.h:70-185, tau 0.97,
// pivot floor 0.25) restated for 7-point rows; the factorisation runs as an
// i+j+k wavefront in FP64 and the two triangular sweeps as the pipelined
// FP32 wavefront of flip_wavefront.cu.  CG (pcgsolver.h:248-302): the
// Laplacian apply, the solution and the residual are double-float (exact
// float pairs, ~48 bits, on the FP32 pipe; this GPU's FP64 rate is ~1/64 of
// FP32) and the dot products are summed in double-float per thread and FP64
// across threads, so the recurrence tracks b - A x to far below the
// tolerance; the FP32 parts (preconditioner, search direction) only steer
// the iteration.  Every 25
// iterations, and whenever the recurrence reports convergence, the residual
// is recomputed as b - A x (iterative refinement), and convergence is
// decided on it, with the reference's test |r|inf <= tol * |b|inf.
#include <algorithm>
#include <cmath>

#include <cooperative_groups.h>
#include <cstring>
#include <string>

#include "../../include/flip3d.h"
#include "flip_device.cuh"

namespace flip {

namespace cg = cooperative_groups;

namespace {

constexpr int TPB = 256;
constexpr int RBLOCKS = 152 * 8;   // grid of the reduction kernels: 8 CTAs of 256 threads per SM (full occupancy)

__device__ __forceinline__ bool sys_cell(const StepConsts &c, const float *phi, int i, int j, int k) {
    if (i < 1 || j < 1 || k < 1 || i > c.I - 2 || j > c.J - 2 || k > c.K - 2) return false;
    return phi[(long long)i + (long long)c.I * ((long long)j + (long long)c.J * k)] < 0.0f;
}

__global__ void k_flags(StepConsts c, const float *phi, uint8_t *fluid, int *fluidFlag, int *levelRange) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    Dims d{c.I, c.J, c.K};
    bool f = false;
    int lv = 0;
    if (t < d.size()) {
        int i, j, k;
        unflatten(t, c.I, c.J, i, j, k);
        f = sys_cell(c, phi, i, j, k);
        fluid[t] = f ? 1 : 0;
        fluidFlag[t] = f ? 1 : 0;
        lv = i + j + k;
    }
    // warp-aggregated min/max/count of the system cells' levels, and their
    // extent in j and k (for the sweep tile orientation)
    unsigned int m = __ballot_sync(0xffffffffu, f);
    if (!m) return;
    int jk[4] = {0x7fffffff, -1, 0x7fffffff, -1};
    if (f) {
        int i, j, k;
        unflatten(t, c.I, c.J, i, j, k);
        jk[0] = jk[1] = j;
        jk[2] = jk[3] = k;
    }
    int lo = f ? lv : 0x7fffffff, hi = f ? lv : -1;
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        jk[0] = min(jk[0], __shfl_xor_sync(0xffffffffu, jk[0], o));
        jk[1] = max(jk[1], __shfl_xor_sync(0xffffffffu, jk[1], o));
        jk[2] = min(jk[2], __shfl_xor_sync(0xffffffffu, jk[2], o));
        jk[3] = max(jk[3], __shfl_xor_sync(0xffffffffu, jk[3], o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&levelRange[0], lo);
        atomicMax(&levelRange[1], hi);
        atomicAdd(&levelRange[2], __popc(m));
        atomicMin(&levelRange[3], jk[0]);
        atomicMax(&levelRange[4], jk[1]);
        atomicMin(&levelRange[5], jk[2]);
        atomicMax(&levelRange[6], jk[3]);
    }
}

// One matrix row in FP64, as _calculateMatrixCoefficientsThread builds it
// (pressuresolver.cpp:723-808).  Off-diagonal entries exist only towards
// neighbours that are rows of the system; a liquid neighbour outside the
// interior contributes neither an entry nor a ghost-fluid term (the
// reference's key map drops it).
__device__ double4_32a row_coeffs(const StepConsts &c, const float *phi, const float *wu, const float *wv,
                              const float *ww, double mf, int i, int j, int k) {
    Dims du{c.I + 1, c.J, c.K}, dv{c.I, c.J + 1, c.K}, dw{c.I, c.J, c.K + 1}, dc{c.I, c.J, c.K};
    double vR = wu[du.idx(i + 1, j, k)], vL = wu[du.idx(i, j, k)];
    double vT = wv[dv.idx(i, j + 1, k)], vB = wv[dv.idx(i, j, k)];
    double vF = ww[dw.idx(i, j, k + 1)], vK = ww[dw.idx(i, j, k)];
    double pc = phi[dc.idx(i, j, k)];
    double diag = (vR + vL + vT + vB + vF + vK) * mf;
    double xp = 0.0, yp = 0.0, zp = 0.0;
    const double maxtheta = 25.0, eps = 1e-9;
    const int nb[6][3] = {{i + 1, j, k}, {i - 1, j, k}, {i, j + 1, k}, {i, j - 1, k}, {i, j, k + 1}, {i, j, k - 1}};
    const double vol[6] = {vR, vL, vT, vB, vF, vK};
#pragma unroll
    for (int q = 0; q < 6; q++) {
        double pn = phi[dc.idx(nb[q][0], nb[q][1], nb[q][2])];
        if (pn < 0.0) {
            if (sys_cell(c, phi, nb[q][0], nb[q][1], nb[q][2])) {
                if (q == 0) xp = -vol[q] * mf;
                else if (q == 2) yp = -vol[q] * mf;
                else if (q == 4) zp = -vol[q] * mf;
            }
        } else {
            double theta = pn / (pc + eps);
            theta = fmax(-maxtheta, fmin(theta, maxtheta));
            diag -= vol[q] * mf * theta;
        }
    }
    return make_double4_32a(fmax(diag, 0.0), xp, yp, zp);
}

// Max of non-negative values over the block, then one atomic per block.
// With nanAsInf a NaN reads as +inf (a residual norm that never passes for
// converged); otherwise NaNs are ignored, as fmax ignores them.
__device__ __forceinline__ void block_max_to(double v, unsigned long long *out, bool nanAsInf = true) {
    __shared__ double sh[32];
    if (v != v) v = nanAsInf ? __longlong_as_double(0x7ff0000000000000ll) : 0.0;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0 && v > 0.0) atomicMax(out, (unsigned long long)__double_as_longlong(v));
    }
}

// RHS (pressuresolver.cpp:580-669; the domain walls do not move) and the rows.
__global__ void k_build(StepConsts c, const float *phi, const float *wu, const float *wv, const float *ww,
                        const float *u, const float *v, const float *w, double mf, PressureBuffers pb) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    Dims d{c.I, c.J, c.K};
    double bmag = 0.0;
    if (t < d.size()) {
        pb.x[t] = make_float2(0.0f, 0.0f);
        pb.r[t] = make_float2(0.0f, 0.0f);
        pb.q[t] = make_float2(0.0f, 0.0f);
        pb.s[t] = 0.0f;
        pb.s2[t] = 0.0f;
        pb.invdiagD[t] = 0.0;
        if (!pb.fluid[t]) {
            pb.Ad[t] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
            pb.A2[2 * t] = pb.A2[2 * t + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            pb.b[t] = 0.0;
        } else {
            int i, j, k;
        unflatten(t, c.I, c.J, i, j, k);
            Dims du{c.I + 1, c.J, c.K}, dv{c.I, c.J + 1, c.K}, dw{c.I, c.J, c.K + 1};
            double vR = wu[du.idx(i + 1, j, k)], vL = wu[du.idx(i, j, k)];
            double vT = wv[dv.idx(i, j + 1, k)], vB = wv[dv.idx(i, j, k)];
            double vF = ww[dw.idx(i, j, k + 1)], vK = ww[dw.idx(i, j, k)];
            double factor = 1.0 / c.dx;
            double div = 0.0;
            div += -factor * vR * (double)u[du.idx(i + 1, j, k)];
            div += factor * vL * (double)u[du.idx(i, j, k)];
            div += -factor * vT * (double)v[dv.idx(i, j + 1, k)];
            div += factor * vB * (double)v[dv.idx(i, j, k)];
            div += -factor * vF * (double)w[dw.idx(i, j, k + 1)];
            div += factor * vK * (double)w[dw.idx(i, j, k)];
            pb.b[t] = div;
            bmag = fabs(div);
            const double4_32a a = row_coeffs(c, phi, wu, wv, ww, mf, i, j, k);
            pb.Ad[t] = a;
            const float4 hi = make_float4((float)a.x, (float)a.y, (float)a.z, (float)a.w);
            pb.A2[2 * t] = hi;
            pb.A2[2 * t + 1] = make_float4((float)(a.x - (double)hi.x), (float)(a.y - (double)hi.y),
                                           (float)(a.z - (double)hi.z), (float)(a.w - (double)hi.w));
        }
    }
    block_max_to(bmag, (unsigned long long *)pb.scal + 2, false);
}

// MIC(0) pivots of one wavefront i+j+k = level, FP64.  For 7-point rows the
// column-oriented elimination of factorModifiedIncompleteColesky0 reduces to:
//   d_c = A_cc - sum over earlier neighbours k (ascending index) of
//         L_ck^2 + 0.97 L_ck (sum of k's other later-neighbour entries L_mk),
//   L_mk = A_mk / sqrt(pivot_k); a pivot below 0.25 A_kk falls back to A_kk.
__device__ __forceinline__ void mic0_cell(const StepConsts &c, const uint8_t *fluid, const double4_32a *Ad, double *invD,
                                          int level, int jj) {
    int nj = c.J - 2;
    int j = 1 + jj % nj, k = 1 + jj / nj;
    int i = level - j - k;
    if (i < 1 || i > c.I - 2) return;
    const long long sy = c.I, sz = (long long)c.I * c.J;
    long long t = i + sy * j + sz * k;
    if (!fluid[t]) return;
    double ad = Ad[t].x;
    double d = ad;
    const long long back[3] = {t - sz, t - sy, t - 1};   // ascending: -z, -y, -x
#pragma unroll
    for (int q = 0; q < 3; q++) {
        long long kk = back[q];
        if (!fluid[kk]) continue;
        double4_32a ak = Ad[kk];
        if (ak.x == 0.0) continue;
        double inv = invD[kk];
        double Lck = (q == 0 ? ak.w : (q == 1 ? ak.z : ak.y)) * inv;
        // k's later neighbours, ascending +x, +y, +z, without c itself
        double miss = 0.0;
        if (q != 2 && fluid[kk + 1]) miss += ak.y * inv;
        if (q != 1 && fluid[kk + sy]) miss += ak.z * inv;
        if (q != 0 && fluid[kk + sz]) miss += ak.w * inv;
        d -= Lck * Lck;
        d -= 0.97 * Lck * miss;
    }
    double inv;
    if (ad == 0.0) inv = 0.0;
    else if (d < 0.25 * ad) inv = 1 / sqrt(ad);
    else inv = 1 / sqrt(d);
    invD[t] = inv;
}

__global__ void k_mic0_level(StepConsts c, const uint8_t *fluid, const double4_32a *Ad, double *invD, int level) {
    int jj = blockIdx.x * blockDim.x + threadIdx.x;
    if (jj < (c.J - 2) * (c.K - 2)) mic0_cell(c, fluid, Ad, invD, level, jj);
}

// All wavefronts lo..hi in one cooperative launch: the cells of a level in
// parallel, a grid-wide barrier between levels (every block is resident, so
// the barrier completes).
__global__ void k_mic0_levels(StepConsts c, const uint8_t *fluid, const double4_32a *Ad, double *invD, int lo, int hi) {
    cg::grid_group grid = cg::this_grid();
    const int np = (c.J - 2) * (c.K - 2);
    for (int lv = lo; lv <= hi; lv++) {
        for (int jj = blockIdx.x * blockDim.x + threadIdx.x; jj < np; jj += gridDim.x * blockDim.x)
            mic0_cell(c, fluid, Ad, invD, lv, jj);
        grid.sync();
    }
}

// The pivot of cell c (mic0_cell) regrouped per earlier neighbour q:
//   L_cq^2 + 0.97 L_cq miss_q = inv_q^2 (a_q^2 + 0.97 a_q (m1_q + m2_q)),
// with a_q the coupling of q to c and m1_q, m2_q q's other later-neighbour
// couplings (0 where mic0_cell skips them).  The bracket depends on the rows
// only; this pass computes it for every cell and earlier neighbour, so a
// level needs three multiply-subtracts and a reciprocal square root.  The
// FP64 results differ from mic0_cell's order in the last bits; the factor
// is used rounded to FP32.
__global__ void k_mic0_weights(StepConsts c, const uint8_t *fluid, const double4_32a *Ad, double *W0, double *W1,
                               double *W2) {
    const long long n = (long long)c.I * c.J * c.K;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    double w[3] = {0.0, 0.0, 0.0};
    if (fluid[t]) {   // interior by construction
        const long long sy = c.I, sz = (long long)c.I * c.J;
        const long long back[3] = {t - sz, t - sy, t - 1};
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const long long kk = back[q];
            if (!fluid[kk]) continue;
            const double4_32a ak = Ad[kk];
            if (ak.x == 0.0) continue;
            const double a = q == 0 ? ak.w : (q == 1 ? ak.z : ak.y);
            const double o1 = q == 2 ? ak.z : ak.y, o2 = q == 0 ? ak.z : ak.w;
            const double m1 = fluid[q == 2 ? kk + sy : kk + 1] ? o1 : 0.0;
            const double m2 = fluid[q == 0 ? kk + sy : kk + sz] ? o2 : 0.0;
            w[q] = a * a + 0.97 * a * (m1 + m2);
        }
    }
    W0[t] = w[0];
    W1[t] = w[1];
    W2[t] = w[2];
}

// The factor as a tiled wavefront, with no grid-wide barrier: a CTA per
// tile of FT x FT (j, k) pencils, tiles taken by ticket in diagonal order
// (a tile only waits on tiles with smaller tickets, which are running or
// done).  Within a tile a level costs one __syncthreads: the -y and -z
// neighbours' pivots of the level before sit in shared memory, the -x one
// in a register.  Across tiles a tile publishes the last level it finished
// every FCH levels (release), and a tile's edge threads read FCH levels of
// the neighbouring pencil's pivots at once, after acquiring its progress.
// Every wait is bounded: past the limit the tile sets *err and all tiles
// that depend on it give up too (the solve reports a device timeout).
// A level is bound by the latency of its FP64 chain (a dependent FP64
// operation takes ~64 cycles on this GPU, rsqrt ~430), not by throughput:
// tiles of 8, 12 and 16 pencils a side time the same.
#ifndef MIC0_FT
#define MIC0_FT 16
#endif
#ifndef MIC0_FCH
#define MIC0_FCH 8
#endif
constexpr int FT = MIC0_FT, FCH = MIC0_FCH;
static_assert(FT * FT >= 32 && FT * FT <= 1024, "a tile is one CTA");
constexpr int FACTOR_DONE = 0x7fffffff;   // progress of a tile with all its levels done

__device__ __forceinline__ int ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int *p, int v) {
    asm volatile("st.release.gpu.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__global__ void __launch_bounds__(FT *FT) k_mic0_tiles(StepConsts c, const uint8_t *fluid, const double4_32a *Ad,
                                                       const double *W0, const double *W1, const double *W2,
                                                       double *invD, int lo, int hi, unsigned int *ticket,
                                                       int *progress, int *err, unsigned int spinLimit) {
    __shared__ double prev[2][FT][FT];
    __shared__ int tileSh, abortSh;
    const int ntj = (c.J - 2 + FT - 1) / FT, ntk = (c.K - 2 + FT - 1) / FT;
    if (threadIdx.x == 0) {
        // ticket -> tile in diagonal order (tj + tk, then tj)
        int q = (int)atomicAdd(ticket, 1u), d = 0;
        for (; d < ntj + ntk - 1; d++) {
            const int n = min(d, ntj - 1) - max(0, d - ntk + 1) + 1;
            if (q < n) break;
            q -= n;
        }
        abortSh = d >= ntj + ntk - 1;   // more CTAs than tiles: the launch is wrong
        if (abortSh) atomicExch(err, 1);
        const int tj = max(0, d - ntk + 1) + q;
        tileSh = tj + ntj * (d - tj);
    }
    __syncthreads();
    if (abortSh) return;
    const int tile = tileSh, tj = tile % ntj, tk = tile / ntj;
    const int a = threadIdx.x % FT, b = threadIdx.x / FT;   // j and k within the tile
    const int j = 1 + tj * FT + a, k = 1 + tk * FT + b;
    const bool mine = j <= c.J - 2 && k <= c.K - 2;
    const int sy = c.I, sz = c.I * c.J;
    // the levels holding cells of this tile, within lo..hi
    const int jhi = min(c.J - 2, 1 + tj * FT + FT - 1), khi = min(c.K - 2, 1 + tk * FT + FT - 1);
    const int lvStart = max(lo, 1 + (1 + tj * FT) + (1 + tk * FT));
    const int lvEnd = min(hi, (c.I - 2) + jhi + khi);
    const int left = tj > 0 ? tile - 1 : -1, down = tk > 0 ? tile - ntj : -1;
    prev[0][b][a] = prev[1][b][a] = 0.0;
    if (threadIdx.x == 0) st_release(&progress[tile], lvStart - 1);   // the levels below hold no cell of the tile
    int cur = 0;
    double own = 0.0;   // this pencil's pivot at the level before (the -x neighbour's)
    for (int lvc = lvStart; lvc <= lvEnd; lvc += FCH) {
        // the chunk's boundary values are the neighbours' levels lvc-1 .. lvc+FCH-2
        if (threadIdx.x == 0) {
            const int need = lvc + FCH - 2;
            const int nbr[2] = {left, down};
            for (int q = 0; q < 2 && !abortSh; q++) {
                if (nbr[q] < 0) continue;
                unsigned int spin = 0;
                while (ld_acquire(&progress[nbr[q]]) < need) {
                    if (++spin >= spinLimit || ld_acquire(err)) {
                        atomicExch(err, 1);
                        abortSh = 1;
                        break;
                    }
                    if (spin > 256) __nanosleep(128);
                }
            }
        }
        __syncthreads();
        if (abortSh) return;
        // the chunk's cells of this pencil are consecutive along i: their
        // rows, flags and weights, and the edge pencils' pivots, load at once
        double bY[FCH], bZ[FCH], pad[FCH], pw0[FCH], pw1[FCH], pw2[FCH];
        bool pcell[FCH];
#pragma unroll
        for (int m = 0; m < FCH; m++) {
            const int i = lvc + m - j - k;
            const bool in = mine && i >= 1 && i <= c.I - 2 && lvc + m <= lvEnd;
            const int t = i + sy * j + sz * k;
            pcell[m] = in && fluid[t];
            pad[m] = pcell[m] ? Ad[t].x : 0.0;
            pw0[m] = pcell[m] ? W0[t] : 0.0;
            pw1[m] = pcell[m] ? W1[t] : 0.0;
            pw2[m] = pcell[m] ? W2[t] : 0.0;
            bY[m] = (pcell[m] && a == 0 && left >= 0) ? __ldcg(invD + t - sy) : 0.0;
            bZ[m] = (pcell[m] && b == 0 && down >= 0) ? __ldcg(invD + t - sz) : 0.0;
        }
#pragma unroll
        for (int m = 0; m < FCH; m++) {
            const int lv = lvc + m;
            if (lv > lvEnd) break;
            double inv = 0.0;
            if (pcell[m]) {
                const int t = (lv - j - k) + sy * j + sz * k;
                const double ad = pad[m];
                const double nz = b > 0 ? prev[cur ^ 1][b - 1][a] : bZ[m];
                const double ny = a > 0 ? prev[cur ^ 1][b][a - 1] : bY[m];
                double d = ad;
                d -= pw0[m] * (nz * nz);
                d -= pw1[m] * (ny * ny);
                d -= pw2[m] * (own * own);
                if (ad == 0.0) inv = 0.0;
                else if (d < 0.25 * ad) inv = rsqrt(ad);
                else inv = rsqrt(d);
                invD[t] = inv;
            }
            prev[cur][b][a] = inv;
            own = inv;
            cur ^= 1;
            __syncthreads();
        }
        if (threadIdx.x == 0) st_release(&progress[tile], min(lvc + FCH - 1, lvEnd));
    }
    if (threadIdx.x == 0) st_release(&progress[tile], FACTOR_DONE);
}

// the FP32 factor rows of the interior cells, into the sweep layout
__global__ void k_mic0_finalize(StepConsts c, SweepLayout g, const uint8_t *fluid, const double4_32a *Ad,
                                const double *invD, float4 *L) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)c.I * c.J * c.K) return;
    int i, j, k;
    unflatten(t, c.I, c.J, i, j, k);
    if (i < 1 || j < 1 || k < 1 || i > c.I - 2 || j > c.J - 2 || k > c.K - 2) return;
    const double inv = invD[t];
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (fluid[t] && inv != 0.0) {
        const double4_32a a = Ad[t];
        v = make_float4((float)inv, (float)(a.y * inv), (float)(a.z * inv), (float)(a.w * inv));
    }
    L[sweep_index(g, i, j, k)] = v;
}

template <class T>
__device__ __forceinline__ T block_sum(T v, T *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    T s = 0;
    if (threadIdx.x == 0)
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) s += sh[q];
    __syncthreads();
    return s;
}


// Each CTA of a reduction takes a ticket once its partial (or atomic) is
// out; the CTA that takes the last one then sees all of them and finishes the
// reduction, and resets the ticket for the next launch.  One launch instead
// of a producer and a one-CTA consumer.
__device__ __forceinline__ bool last_cta(unsigned int *ticket) {
    __shared__ int amLast;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        amLast = atomicAdd(ticket, 1u) == gridDim.x - 1;
        if (amLast) {
            *ticket = 0u;
            __threadfence();
        }
    }
    __syncthreads();
    return amLast;
}
// Sum of the launch's block partials in a fixed order (deterministic);
// thread 0 holds the result.
__device__ __forceinline__ double sum_partials_fixed(const double *partials, int n, double *sh) {
    double v = 0.0;
    for (int q = threadIdx.x; q < n; q += blockDim.x) v += __ldcg(partials + q);
    return block_sum(v, sh);
}
__device__ __forceinline__ double bits_to_resid(const unsigned long long *p) {
    return __longlong_as_double((long long)__ldcg(p));
}

// The reductions below run on a fixed grid per context (nPartials CTAs,
// pressure_partials_for) with grid-stride loops: each thread sums its rows
// in a fixed order, each CTA writes one partial, and the last CTA adds the
// partials in a fixed order, so every sum is deterministic and the FP64
// reduction work is per thread, not per row.

// the rows of the system as a list: flat index and sweep-layout index
__global__ void k_compact_rows(StepConsts c, SweepLayout g, const uint8_t *fluid, const int *pos, int *idx, int *sk) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)c.I * c.J * c.K || !fluid[t]) return;
    int i, j, k;
    unflatten(t, c.I, c.J, i, j, k);
    const int e = pos[t];
    idx[e] = (int)t;
    sk[e] = (int)sweep_index(g, i, j, k);
}

// Double-float arithmetic on the FP32 pipe (this GPU's FP64 rate is ~1/64
// of FP32): a coefficient a = hi + lo (floats, exact to 48 bits) times an
// FP32 s is hi*s exactly as a rounded product plus its FMA-recovered error,
// plus lo*s; sums carry their rounding errors in a second float (Knuth's
// TwoSum).  A 7-term row sum is exact to ~2^-48 of its terms, where FP64 is
// exact to ~2^-53.
__device__ __forceinline__ float2 df_from(double v) {
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}
__device__ __forceinline__ double df_to(float2 v) { return (double)v.x + (double)v.y; }
// (h, l) with h = fl(h + l): the pair in normalised form (|l| <= ulp(h) / 2)
__device__ __forceinline__ float2 df_norm(float h, float l) {
    const float s = __fadd_rn(h, l);
    return make_float2(s, __fsub_rn(l, __fsub_rn(s, h)));
}
// a + b for pairs: TwoSum of the leading parts, the rest added to the error
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    const float t = __fadd_rn(a.x, b.x);
    const float bb = __fsub_rn(t, a.x);
    const float err = __fadd_rn(__fsub_rn(a.x, __fsub_rn(t, bb)), __fsub_rn(b.x, bb));
    return df_norm(t, __fadd_rn(err, __fadd_rn(a.y, b.y)));
}
// f * v for a float f and a pair v: the leading product exact as its
// rounded value plus its FMA-recovered error
__device__ __forceinline__ float2 df_scale(float f, float2 v) {
    const float ph = __fmul_rn(f, v.x);
    const float pl = __fmaf_rn(f, v.y, __fmaf_rn(f, v.x, -ph));
    return make_float2(ph, pl);
}
__device__ __forceinline__ void df_mul_add(float ah, float al, float sv, float &sh, float &sl) {
    const float ph = __fmul_rn(ah, sv);
    float pl = __fmaf_rn(ah, sv, -ph);   // exact error of ah * sv
    pl = __fmaf_rn(al, sv, pl);
    const float t = __fadd_rn(sh, ph);
    const float bb = __fsub_rn(t, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bb)), __fsub_rn(ph, bb));   // exact error of sh + ph
    sl = __fadd_rn(sl, __fadd_rn(err, pl));
    sh = t;
}

// s = z + beta s (pcgsolver.h:295-298, beta rounded to float) fused with
// q = A s over the rows in double-float, stored as a pair; s.q summed in
// double-float per thread and in FP64 across threads.  The new s of a row's
// stencil is formed from the previous iteration's buffer sIn (so no row
// reads a value another thread is writing) and the row's own goes to sOut.
// z is read in cell order (zc, written by the z.r pass before it).  In the
// first iteration beta = 0 and sIn = 0, so s = z.  A neighbour that
// is not a row couples with 0 and takes s = 0.  The last CTA sums s.q and
// sets alpha = rho / s.q, rounded to float as BLAS::addScaled takes it
// (blaswrapper.h:129-158), and clears the iteration's residual norms.
__global__ void k_spmv_s(StepConsts c, const int *__restrict__ rows,
                         const int *nRows, const float4 *__restrict__ A2, const float *__restrict__ z,
                         const float *__restrict__ sIn, float *__restrict__ sOut, float2 *__restrict__ q,
                         double *partials, double *scal, unsigned long long *rmaxBits, PcgCtl *ctl) {
    __shared__ double sh[32];
    if (ctl->done) return;
    const int n = *nRows;
    const float beta = (float)scal[5];   // exact: beta is a float value
    const long long sy = c.I, sz = (long long)c.I * c.J;
    float2 dot = make_float2(0.0f, 0.0f);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const long long t = rows[e];
        const float4 hi = A2[2 * t], lo = A2[2 * t + 1];
        const float4 hxm = A2[2 * (t - 1)], lxm = A2[2 * (t - 1) + 1];
        const float4 hym = A2[2 * (t - sy)], lym = A2[2 * (t - sy) + 1];
        const float4 hzm = A2[2 * (t - sz)], lzm = A2[2 * (t - sz) + 1];
        // the search direction over the stencil's rows
        auto snew = [&](bool row, long long tn) {
            return row ? __fmaf_rn(beta, sIn[tn], z[tn]) : 0.0f;
        };
        const float st = snew(true, t);
        const float sxp = snew(hi.y != 0.0f || lo.y != 0.0f, t + 1);
        const float syp = snew(hi.z != 0.0f || lo.z != 0.0f, t + sy);
        const float szp = snew(hi.w != 0.0f || lo.w != 0.0f, t + sz);
        const float sxm = snew(hxm.y != 0.0f || lxm.y != 0.0f, t - 1);
        const float sym = snew(hym.z != 0.0f || lym.z != 0.0f, t - sy);
        const float szm = snew(hzm.w != 0.0f || lzm.w != 0.0f, t - sz);
        sOut[t] = st;
        float accH = 0.0f, accL = 0.0f;
        df_mul_add(hi.x, lo.x, st, accH, accL);
        df_mul_add(hi.y, lo.y, sxp, accH, accL);
        df_mul_add(hi.z, lo.z, syp, accH, accL);
        df_mul_add(hi.w, lo.w, szp, accH, accL);
        df_mul_add(hxm.y, lxm.y, sxm, accH, accL);
        df_mul_add(hym.z, lym.z, sym, accH, accL);
        df_mul_add(hzm.w, lzm.w, szm, accH, accL);
        const float2 qt = df_norm(accH, accL);
        q[t] = qt;
        dot = df_add(dot, df_scale(st, qt));
    }
    double b = block_sum(df_to(dot), sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = b;
    if (last_cta(&ctl->ticket[0])) {
        const double sq = sum_partials_fixed(partials, gridDim.x, sh);
        if (threadIdx.x == 0) {
            scal[0] = sq;
            scal[4] = (double)(float)(scal[3] / sq);
            rmaxBits[0] = 0ull;
            rmaxBits[1] = 0ull;
        }
    }
}

// rho_new = z.r.  The last CTA sums it; inside the loop (inLoop) it also
// sets beta = rho_new / rho as float (pcgsolver.h:295-298) and ends the
// iteration: rho = rho_new, next iteration index.  Each row's z, gathered
// from the sweep layout, is also stored in cell order, so that the SpMV's
// stencil reads of z are coalesced.
__global__ void k_dot_zr(const int *__restrict__ rows, const int *__restrict__ rowsSk, const int *nRows,
                         const float *__restrict__ z, float *__restrict__ zc, const float2 *__restrict__ r,
                         double *partials, double *scal,
                         PcgCtl *ctl, int inLoop) {
    __shared__ double sh[32];
    if (ctl->done) return;
    const int n = *nRows;
    float2 dot = make_float2(0.0f, 0.0f);   // double-float per thread, FP64 across threads
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int t = rows[e];
        const float zt = z[rowsSk[e]];
        zc[t] = zt;   // z in cell order, where the SpMV reads its stencil
        dot = df_add(dot, df_scale(zt, r[t]));
    }
    double s = block_sum(df_to(dot), sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
    if (last_cta(&ctl->ticket[1])) {
        const double zr = sum_partials_fixed(partials, gridDim.x, sh);
        if (threadIdx.x == 0) {
            scal[1] = zr;
            if (inLoop) {
                scal[5] = scal[3] != 0.0 ? (double)(float)(zr / scal[3]) : 0.0;
                ctl->it += 1;
            }
            scal[3] = zr;
        }
    }
}

// The reference's convergence test |r|inf <= tol |b|inf (pcgsolver.h:
// 263-288) on the device, by the last CTA of the kernel that produced the
// norm.  On the iterations where r is recomputed as b - A x (every 25th)
// that norm decides; otherwise a pass of the recurrence's norm is only a
// claim, which the recompute of b - A x then settles (final).
__device__ __forceinline__ void convergence_test(PcgCtl *ctl, double resid, double ptol, bool final) {
    ctl->resid = resid;
    ctl->claim = 0;
    if (resid <= ptol) {
        if (final) {
            ctl->done = 1;
            ctl->iters = ctl->it + 1;
        } else {
            ctl->claim = 1;
        }
    }
}

// x += alpha s, r -= alpha q with alpha = rho / s.q passed on as float, as
// BLAS::addScaled(float alpha, ...) does (blaswrapper.h:129-158); |r|inf,
// tested by the last CTA except on the iterations of the periodic recompute
__global__ void k_update_xr(const int *__restrict__ rows, const int *__restrict__ rowsSk, const int *nRows,
                            float2 *__restrict__ x, float2 *__restrict__ r, float *__restrict__ rf,
                            const float *__restrict__ s, const float2 *__restrict__ q, const double *scal,
                            unsigned long long *rmaxBits, PcgCtl *ctl) {
    if (ctl->done) return;
    const int n = *nRows;
    const float alpha = (float)scal[4];   // exact: alpha is a float value
    float m = 0.0f;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int t = rows[e];
        x[t] = df_add(x[t], df_scale(alpha, make_float2(s[t], 0.0f)));   // alpha s is exact as a pair
        const float2 rv = df_add(r[t], df_scale(-alpha, q[t]));
        r[t] = rv;
        rf[rowsSk[e]] = rv.x;   // normalised: the pair rounded to float
        const float av = fabsf(rv.x);
        m = (av != av || av > m) ? av : m;   // a NaN sticks
    }
    block_max_to((double)m, rmaxBits);
    if (last_cta(&ctl->ticket[2]) && threadIdx.x == 0 && (ctl->it + 1) % 25 != 0)
        convergence_test(ctl, bits_to_resid(rmaxBits), scal[6], false);
}

// r = b - A x (residual replacement); |r|inf, which the last CTA tests as
// final.  Inside the loop it runs only when needed: on every 25th iteration
// (pcgsolver.h's periodic recompute, here before the test) and when the
// recurrence just claimed convergence (a claim is only made on the other
// iterations, so one launch serves both); never once converged.
__global__ void k_true_residual(StepConsts c, const int *__restrict__ rows, const int *__restrict__ rowsSk,
                                const int *nRows, const double4_32a *__restrict__ Ad, const double *__restrict__ b,
                                const float2 *__restrict__ x, float2 *__restrict__ r, float *__restrict__ rf,
                                unsigned long long *rmaxBits, const double *scal, PcgCtl *ctl,
                                unsigned int *sweepTicket) {
    if (blockIdx.x == 0 && threadIdx.x == 0) sweep_prep(sweepTicket);   // for the sweep pair that follows
    if (ctl->done) return;
    if ((ctl->it + 1) % 25 != 0 && !ctl->claim) return;
    const int n = *nRows;
    const long long sy = c.I, sz = (long long)c.I * c.J;
    double m = 0.0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const long long t = rows[e];
        const double4_32a a = Ad[t];
        double ax = a.x * df_to(x[t]);
        ax = fma(a.y, df_to(x[t + 1]), ax);
        ax = fma(a.z, df_to(x[t + sy]), ax);
        ax = fma(a.w, df_to(x[t + sz]), ax);
        ax = fma(Ad[t - 1].y, df_to(x[t - 1]), ax);
        ax = fma(Ad[t - sy].z, df_to(x[t - sy]), ax);
        ax = fma(Ad[t - sz].w, df_to(x[t - sz]), ax);
        const double rv = b[t] - ax;
        const float2 rp = df_from(rv);
        r[t] = rp;
        rf[rowsSk[e]] = rp.x;
        const double av = fabs(rv);
        m = (av != av || av > m) ? av : m;
    }
    block_max_to(m, rmaxBits);
    if (last_cta(&ctl->ticket[3]) && threadIdx.x == 0) convergence_test(ctl, bits_to_resid(rmaxBits), scal[6], true);
}

// r = b (and its FP32 copy in the sweep layout), x = 0, |b|inf
__global__ void k_init_r(StepConsts c, SweepLayout g, const double *b, float2 *r, float *rf, float2 *x,
                         unsigned long long *rmaxBits, unsigned int *sweepTicket) {
    const long long n = (long long)c.I * c.J * c.K;
    if (blockIdx.x == 0 && threadIdx.x == 0) sweep_prep(sweepTicket);   // for the first sweep pair
    double m = 0.0;
#pragma unroll 4
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        r[t] = df_from(b[t]);
        x[t] = make_float2(0.0f, 0.0f);
        int i, j, k;
    unflatten(t, c.I, c.J, i, j, k);
        if (i >= 1 && j >= 1 && k >= 1 && i <= c.I - 2 && j <= c.J - 2 && k <= c.K - 2)
            rf[sweep_index(g, i, j, k)] = (float)b[t];
        double av = fabs(b[t]);
        m = (av != av || av > m) ? av : m;
    }
    block_max_to(m, rmaxBits);
}

__global__ void k_x_to_float(long long n, const float2 *x, float *p) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) p[t] = (float)df_to(x[t]);
}

// _applyPressureToVelocityFieldThread (pressuresolver.cpp:896-1046) without
// surface tension.  Liquid means phi < 0 over all cells (FluidMaterialGrid,
// :849-858); the faces i == 0 and i == I-1 (and the v/w analogues) are
// skipped as the reference skips them.
__global__ void k_apply_pressure(StepConsts c, const float *phi, const float *wu, const float *wv, const float *ww,
                                 const float *P, float factor, float *u, float *v, float *w, uint8_t *vu,
                                 uint8_t *vv, uint8_t *vw) {
    long long nu = (long long)(c.I + 1) * c.J * c.K, nv = (long long)c.I * (c.J + 1) * c.K;
    long long nw = (long long)c.I * c.J * (c.K + 1);
    long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nu + nv + nw) return;
    int dir = f < nu ? 0 : (f < nu + nv ? 1 : 2);
    long long l = dir == 0 ? f : (dir == 1 ? f - nu : f - nu - nv);
    int ni = c.I + (dir == 0), nj = c.J + (dir == 1);
    int i, j, k;
    unflatten(l, ni, nj, i, j, k);
    float *G = dir == 0 ? u : (dir == 1 ? v : w);
    uint8_t *V = dir == 0 ? vu : (dir == 1 ? vv : vw);
    const float *W = dir == 0 ? wu : (dir == 1 ? wv : ww);
    V[l] = 0;
    int g = dir == 0 ? i : (dir == 1 ? j : k);
    int gmax = dir == 0 ? c.I : (dir == 1 ? c.J : c.K);
    if (g == 0 || g == gmax - 1) return;
    Dims dc{c.I, c.J, c.K};
    int ai = i - (dir == 0), aj = j - (dir == 1), ak = k - (dir == 2);
    bool fb = dc.in(i, j, k) && phi[dc.idx(i, j, k)] < 0.0f;
    bool fa = phi[dc.idx(ai, aj, ak)] < 0.0f;
    bool border = (g == gmax) ? fa : (fb || fa);
    if (!(W[l] > 0.0f && border)) {
        G[l] = 0.0f;
        return;
    }
    float p1, p2;
    const float eps = 1e-6f;
    const double maxtheta = 25.0;
    if (fa && fb) {
        p1 = P[dc.idx(ai, aj, ak)];
        p2 = P[dc.idx(i, j, k)];
    } else {
        float phi1 = phi[dc.idx(ai, aj, ak)], phi2 = phi[dc.idx(i, j, k)];
        if (fa) {
            float tp = (float)fmax(-maxtheta, fmin((double)__fdiv_rn(phi2, __fadd_rn(phi1, eps)), maxtheta));
            p1 = P[dc.idx(ai, aj, ak)];
            p2 = __fmul_rn(tp, p1);
        } else {
            float tp = (float)fmax(-maxtheta, fmin((double)__fdiv_rn(phi1, __fadd_rn(phi2, eps)), maxtheta));
            p2 = P[dc.idx(i, j, k)];
            p1 = __fmul_rn(tp, p2);
        }
    }
    G[l] = __fadd_rn(G[l], __fmul_rn(-factor, __fsub_rn(p2, p1)));
    V[l] = 1;
}

int cuda_fail(cudaError_t e, const char *what, std::string *msg) {
    if (msg) *msg = std::string("pressure solve: ") + what + ": " + cudaGetErrorString(e);
    return FLIP_E_CUDA;
}

}  // namespace

int mic0_factor_tiles(int J, int K) { return std::max(1, (J - 2 + FT - 1) / FT) * std::max(1, (K - 2 + FT - 1) / FT); }
// One reduction CTA per `cellsPerCta` grid cells (4096 by default), at most
// RBLOCKS.  A liquid fills a fraction of the grid, so a thread takes a few
// rows; a smaller grid spares the GPU's CTA dispatch, which many scenes
// running at once share.
int pressure_partials_for(int I, int J, int K, int cellsPerCta) {
    static_assert(RBLOCKS == PCG_MAX_PARTIALS, "the partials buffer holds RBLOCKS sums");
    return std::min((int)div_up((long long)I * J * K, std::max(cellsPerCta, 256)), RBLOCKS);
}

#define PCK(call)                                               \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call, errMsg); \
    } while (0)

// MIC(0) factor of the rows Ad over the cells flagged in `fluid`, whose
// levels i+j+k lie in lo..hi: the inverse pivots invD (FP64).  The tiled
// wavefront runs where it launches; otherwise one cooperative launch over all
// levels, else one launch per level.  W0..W2: n doubles each of scratch;
// progress: mic0_factor_tiles ints; err: set when a bounded wait gave up.
void mic0_factor(const StepConsts &c, const uint8_t *fluid, const double4_32a *Ad, double *invD, double *W0,
                 double *W1, double *W2, int *progress, unsigned int *ticket, int *err, unsigned int spinLimit,
                 int lo, int hi, cudaStream_t s) {
    const long long n = (long long)c.I * c.J * c.K;
    const unsigned nb = div_up(n, TPB);
    const int np = (c.J - 2) * (c.K - 2);
    const int ntiles = mic0_factor_tiles(c.J, c.K);
    cudaMemsetAsync(progress, 0xff, ntiles * sizeof(int), s);
    cudaMemsetAsync(ticket, 0, sizeof(unsigned int), s);
    { FLIP_COUNT(1); k_mic0_weights<<<nb, TPB, 0, s>>>(c, fluid, Ad, W0, W1, W2); }
    FLIP_COUNT(1);
    k_mic0_tiles<<<ntiles, FT * FT, 0, s>>>(c, fluid, Ad, W0, W1, W2, invD, lo, hi, ticket, progress, err, spinLimit);
    if (cudaGetLastError() == cudaSuccess) return;
    int dev = 0, coop = 0, perSM = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_mic0_levels, TPB, 0);
    if (coop && perSM > 0) {
        StepConsts c_ = c;
        int lo_ = lo, hi_ = hi;
        void *args[] = {&c_, &fluid, &Ad, &invD, &lo_, &hi_};
        const int grid = std::max(1, std::min((int)div_up(np, TPB), perSM * sms));
        FLIP_COUNT(1);
        if (cudaLaunchCooperativeKernel((const void *)k_mic0_levels, grid, TPB, args, 0, s) == cudaSuccess) return;
        cudaGetLastError();
    }
    for (int lv = lo; lv <= hi; lv++) {
        FLIP_COUNT(1);
        k_mic0_level<<<div_up(np, TPB), TPB, 0, s>>>(c, fluid, Ad, invD, lv);
    }
}

// The condition of the device-side loop over batches of PCG iterations: one
// more batch while the solve has not converged, no wavefront has given up
// and fewer than maxBatches batches have run (so the loop always ends).
__global__ void k_pcg_loop(cudaGraphConditionalHandle h, PcgCtl *ctl, const int *err) {
    const int ran = ctl->batches + 1;
    ctl->batches = ran;
    const bool more = !ctl->done && !*(volatile const int *)err && ran < ctl->maxBatches;
    cudaGraphSetConditional(h, more ? 1u : 0u);
}

int pressure_project(const StepConsts &c, const PressureArgs &a, PressureBuffers &pb, SweepState &sw,
                     PressureMail *mail, cudaStream_t s, PressureResult *res, std::string *errMsg) {
    const long long n = (long long)c.I * c.J * c.K;
    const unsigned nb = div_up(n, TPB);
    const unsigned rb = (unsigned)pb.nPartials;   // reduction grid
    const double mf = a.dt / (c.dx * c.dx);
    res->iterations = 0;
    res->residual = 0.0;
    res->applied = false;
    res->cells = 0;
    auto sync = [&]() -> cudaError_t {
        FLIP_SYNC_COUNT();
        cudaError_t e = cudaStreamSynchronize(s);
        return e != cudaSuccess ? e : cudaGetLastError();
    };

    static const int lr[8] = {0x7fffffff, -1, 0, 0x7fffffff, -1, 0x7fffffff, -1, 0};
    std::memcpy(mail->levelRange, lr, sizeof(lr));
    PCK(cudaMemcpyAsync(pb.levelRange, mail->levelRange, sizeof(lr), cudaMemcpyHostToDevice, s));
    PCK(cudaMemsetAsync(pb.scal, 0, 8 * sizeof(double), s));
    { FLIP_COUNT(1); k_flags<<<nb, TPB, 0, s>>>(c, a.phi, pb.fluid, pb.fluidFlag, pb.levelRange); }
    { FLIP_COUNT(1); k_build<<<nb, TPB, 0, s>>>(c, a.phi, a.wu, a.wv, a.ww, a.u, a.v, a.w, mf, pb); }
    PCK(cudaMemcpyAsync(mail->levelRange, pb.levelRange, 7 * sizeof(int), cudaMemcpyDeviceToHost, s));
    PCK(cudaMemcpyAsync(&mail->bmax, pb.scal + 2, sizeof(double), cudaMemcpyDeviceToHost, s));
    PCK(sync());
    if (a.dumpRhs) PCK(cudaMemcpy(a.dumpRhs, pb.b, n * sizeof(double), cudaMemcpyDeviceToHost));
    const int lo = mail->levelRange[0], hi = mail->levelRange[1];
    res->cells = mail->levelRange[2];
    const double bmax = mail->bmax;
    if (hi < lo || bmax < a.tol) {   // no system, or nothing to project (pressuresolver.cpp:53-56)
        if (a.dumpPressure) std::memset(a.dumpPressure, 0, n * sizeof(float));
        return FLIP_OK;
    }
    const double ptol = fmax(a.tol, 1e-30) * bmax;
    if (sw.xchgWords < sweep_exchange_words(c.I, c.J, c.K)) {   // the sweeps' exchange array must cover every step
        if (errMsg) *errMsg = "sweep exchange array smaller than the grid needs";
        return FLIP_E_RUNTIME;
    }
    // Sweep tile orientation for this solve: the one whose tiles the rows'
    // extent crosses with the shorter chain of hops.  A hop across the lane
    // axis delays the next tile by about SL TJ + chunk + handoff steps, across
    // the warp axis by about SW TK + chunk + handoff.
    {
        const int jlo = mail->levelRange[3], jhi = mail->levelRange[4];
        const int klo = mail->levelRange[5], khi = mail->levelRange[6];
        auto hops = [](int lo_, int hi_, int w) { return (hi_ - 1) / w - (lo_ - 1) / w; };
        const int lagA = SWEEP_SL * SWEEP_TJ + 8 + 14, lagB = SWEEP_SW * SWEEP_TK + 8 + 14;
        const long long cost0 = (long long)hops(jlo, jhi, SWEEP_TJ) * lagA + (long long)hops(klo, khi, SWEEP_TK) * lagB;
        const long long cost1 = (long long)hops(klo, khi, SWEEP_TJ) * lagA + (long long)hops(jlo, jhi, SWEEP_TK) * lagB;
        int want = cost1 < cost0 ? 1 : (cost0 < cost1 ? 0 : pb.sl.swap);
        if (a.sweepOrientation == 0 || a.sweepOrientation == 1) want = a.sweepOrientation;
        if (want != pb.sl.swap) {
            pb.sl = sweep_layout(c.I, c.J, c.K, want);
            // entries that hold no interior cell in the new orientation must read zero
            PCK(cudaMemsetAsync(pb.L, 0, pb.nsl * sizeof(float4), s));
            PCK(cudaMemsetAsync(pb.rf, 0, pb.nsl * sizeof(float), s));
            PCK(cudaMemsetAsync(pb.z, 0, pb.nsl * sizeof(float), s));
        }
    }
    // the rows as a list in cell order (a scan keeps it deterministic)
    launch_scan_cells(pb.fluidFlag, (int)n, pb.fluidPos, pb.fluidScan, pb.nFluid, s);
    { FLIP_COUNT(1); k_compact_rows<<<nb, TPB, 0, s>>>(c, pb.sl, pb.fluid, pb.fluidPos, pb.fluidIdx, pb.fluidSk); }

    // MIC(0) factor; the pivot weights go to q, r and x (as FP64 arrays),
    // which the loop set-up rewrites
    mic0_factor(c, pb.fluid, pb.Ad, pb.invdiagD, reinterpret_cast<double *>(pb.q), reinterpret_cast<double *>(pb.r),
                reinterpret_cast<double *>(pb.x), pb.factorProgress, pb.factorTicket, sw.err,
                sw.spinLimit ? sw.spinLimit : DEFAULT_SPIN_LIMIT, lo, hi, s);
    { FLIP_COUNT(1); k_mic0_finalize<<<nb, TPB, 0, s>>>(c, pb.sl, pb.fluid, pb.Ad, pb.invdiagD, pb.L); }
    launch_sweep_ranges(c, pb.sl, pb.fluid, sw, s);

    unsigned long long *rmax = pb.rmaxBits;
    SweepTiming *tm = a.sweepTiming;
    // sweep pairs timed but not yet added: event pair index q
    auto tally_pair = [&](int q) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, tm->ev[2 * q], tm->ev[2 * q + 1]) == cudaSuccess) {
            tm->ms += ms;
            tm->launches += 2;
            tm->cellSweeps += 2LL * res->cells;
        } else {
            cudaGetLastError();   // a pair that was not recorded is not an error of the solve
        }
    };
    bool capturing = false;
    // inside a capture the events become graph nodes that record on every replay
    auto record = [&](cudaEvent_t e) {
        if (capturing) cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
        else cudaEventRecord(e, s);
    };
    // z = M^-1 r, then rho_new = z.r; with `timed` the sweeps sit between
    // event pair q (recorded as graph nodes when captured)
    auto precondition = [&](int q, bool timed) {
        if (timed) record(tm->ev[2 * q]);
        launch_sweeps(c, pb.sl, pb.L, pb.rf, pb.z, sw, &pb.ctl->done, s, true);   // prepared by the kernel before
        if (timed) record(tm->ev[2 * q + 1]);
        { FLIP_COUNT(1); k_dot_zr<<<rb, TPB, 0, s>>>(pb.fluidIdx, pb.fluidSk, pb.nFluid, pb.z, pb.zc, pb.r, pb.partials, pb.scal, pb.ctl, q > 0); }
    };
    // one PCG iteration (pcgsolver.h:263-300); every launch is the same for
    // every iteration but the search direction's two buffers, which swap
    // roles each iteration (a batch of PCG_BATCH, an even count, ends where
    // it began); the iteration index lives on the device
    int sPar = 0;
    auto iteration = [&](int k, bool timed) {
        float *sIn = sPar ? pb.s2 : pb.s, *sOut = sPar ? pb.s : pb.s2;
        { FLIP_COUNT(1); k_spmv_s<<<rb, TPB, 0, s>>>(c, pb.fluidIdx, pb.nFluid, pb.A2, pb.zc, sIn, sOut, pb.q, pb.partials, pb.scal, rmax, pb.ctl); }
        { FLIP_COUNT(1); k_update_xr<<<rb, TPB, 0, s>>>(pb.fluidIdx, pb.fluidSk, pb.nFluid, pb.x, pb.r, pb.rf, sOut, pb.q, pb.scal, rmax, pb.ctl); }
        { FLIP_COUNT(1); k_true_residual<<<rb, TPB, 0, s>>>(c, pb.fluidIdx, pb.fluidSk, pb.nFluid, pb.Ad, pb.b, pb.x, pb.r, pb.rf, rmax + 1, pb.scal, pb.ctl, sw.ticket); }
        precondition(1 + k, timed);
        sPar ^= 1;
    };
    static_assert(PCG_BATCH % 2 == 0, "a batch must leave the search direction in the buffer it started from");

    mail->ptol = ptol;
    PCK(cudaMemsetAsync(pb.ctl, 0, sizeof(PcgCtl), s));
    PCK(cudaMemsetAsync(rmax, 0, 2 * sizeof(unsigned long long), s));
    PCK(cudaMemcpyAsync(pb.scal + 6, &mail->ptol, sizeof(double), cudaMemcpyHostToDevice, s));
    sweep_epoch_guard(c, sw, 2, s);
    { FLIP_COUNT(1); k_init_r<<<rb, TPB, 0, s>>>(c, pb.sl, pb.b, pb.r, pb.rf, pb.x, rmax, sw.ticket); }
    precondition(0, tm != nullptr);
    PCK(cudaMemcpyAsync(&mail->rho, pb.scal + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
    PCK(cudaMemcpyAsync(&mail->sweepErr, sw.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    PCK(sync());
    if (tm) tally_pair(0);
    const double rho0 = mail->rho;
    bool ok = false;
    int iterations = 0;
    double resid = bmax;
    int sweepErr = mail->sweepErr;   // the factor's or the first sweep's bounded wait gave up
    if (!sweepErr && !(rho0 == 0 || rho0 != rho0)) {
        // Iterations go to the device PCG_BATCH at a time, as one CUDA graph
        // (captured on first use, per context): the convergence test runs
        // there and the kernels of iterations after convergence return at
        // once.  Untimed, the full batches run inside a device-side loop (a
        // conditional WHILE node whose body is a batch and k_pcg_loop), so
        // the host launches the solve once and waits once; timed, or where
        // the loop cannot be built, the host reads the outcome once per
        // batch.  The iterations after the last full batch run eagerly.
        const int gi = tm ? 1 : 0, go = pb.sl.swap;
        int it0 = 0;
        const int maxBatches = a.maxIter / PCG_BATCH;
        if (!tm && !pb.noGraphs && !pb.noLoopGraph && maxBatches > 0) {
            sweep_epoch_guard(c, sw, 2LL * PCG_BATCH * maxBatches, s);
            if (!pb.loopGraph[go]) {
                long long &counter = launch_counter();
                const long long before = counter;
                const unsigned int epochBefore = sw.epoch;
                cudaGraph_t graph = nullptr;
                cudaGraphConditionalHandle handle{};
                bool built = false;
                if (cudaGraphCreate(&graph, 0) == cudaSuccess &&
                    cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault) == cudaSuccess) {
                    cudaGraphNodeParams cp{};
                    cp.type = cudaGraphNodeTypeConditional;
                    cp.conditional.handle = handle;
                    cp.conditional.type = cudaGraphCondTypeWhile;
                    cp.conditional.size = 1;
                    cudaGraphNode_t node;
                    if (cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp) == cudaSuccess &&
                        cudaStreamBeginCaptureToGraph(s, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                      cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                        capturing = true;
                        for (int k = 0; k < PCG_BATCH; k++) iteration(k, false);
                        { FLIP_COUNT(1); k_pcg_loop<<<1, 1, 0, s>>>(handle, pb.ctl, sw.err); }
                        capturing = false;
                        cudaGraph_t body = nullptr;
                        built = cudaStreamEndCapture(s, &body) == cudaSuccess &&
                                cudaGraphInstantiate(&pb.loopGraph[go], graph, 0) == cudaSuccess;
                    }
                }
                if (graph) cudaGraphDestroy(graph);
                if (!built) {
                    cudaGetLastError();   // no device-side loop here: batches from the host
                    pb.loopGraph[go] = nullptr;
                    pb.noLoopGraph = true;
                }
                pb.loopKernels[go] = counter - before;
                counter = before;   // counted when run
                sw.epoch = epochBefore;
            }
            if (pb.loopGraph[go]) {
                mail->maxBatches = maxBatches;
                PCK(cudaMemcpyAsync(&pb.ctl->maxBatches, &mail->maxBatches, sizeof(int), cudaMemcpyHostToDevice, s));
                PCK(cudaGraphLaunch(pb.loopGraph[go], s));
                PCK(cudaMemcpyAsync(&mail->ctl, pb.ctl, sizeof(PcgCtl), cudaMemcpyDeviceToHost, s));
                PCK(cudaMemcpyAsync(&mail->sweepErr, sw.err, sizeof(int), cudaMemcpyDeviceToHost, s));
                PCK(sync());
                const int ran = mail->ctl.batches;
                launch_counter() += ran * pb.loopKernels[go];
                sw.epoch += 2u * PCG_BATCH * (unsigned int)ran;
                sweepErr = mail->sweepErr;
                resid = mail->ctl.resid;
                if (!sweepErr && mail->ctl.done) {
                    ok = true;
                    iterations = mail->ctl.iters;
                }
                it0 = ran * PCG_BATCH;
            }
        }
        while (!ok && !sweepErr && it0 < a.maxIter) {
            const int nit = std::min(PCG_BATCH, a.maxIter - it0);
            sweep_epoch_guard(c, sw, 2LL * nit, s);
            if (nit == PCG_BATCH && !pb.batchGraph[gi][go] && !pb.noGraphs) {
                long long &counter = launch_counter();
                const long long before = counter;
                const unsigned int epochBefore = sw.epoch;
                if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                    cudaGetLastError();   // e.g. the legacy default stream: no graphs, launch eagerly
                    pb.noGraphs = true;
                } else {
                    cudaGraph_t graph = nullptr;
                    capturing = true;
                    for (int k = 0; k < PCG_BATCH; k++) iteration(k, tm != nullptr);
                    capturing = false;
                    PCK(cudaStreamEndCapture(s, &graph));
                    cudaError_t e = cudaGraphInstantiate(&pb.batchGraph[gi][go], graph, 0);
                    cudaGraphDestroy(graph);
                    PCK(e);
                    pb.batchKernels[gi][go] = counter - before;
                    counter = before;   // counted when replayed
                    sw.epoch = epochBefore;
                }
            }
            if (nit == PCG_BATCH && pb.batchGraph[gi][go]) {
                PCK(cudaGraphLaunch(pb.batchGraph[gi][go], s));
                launch_counter() += pb.batchKernels[gi][go];
                sw.epoch += 2 * PCG_BATCH;
            } else {
                for (int k = 0; k < nit; k++) iteration(k, tm != nullptr);
            }
            PCK(cudaMemcpyAsync(&mail->ctl, pb.ctl, sizeof(PcgCtl), cudaMemcpyDeviceToHost, s));
            PCK(cudaMemcpyAsync(&mail->sweepErr, sw.err, sizeof(int), cudaMemcpyDeviceToHost, s));
            PCK(sync());
            sweepErr = mail->sweepErr;
            resid = mail->ctl.resid;
            if (tm)   // the sweep pairs that ran: all before convergence
                for (int k = 0; k < nit; k++)
                    if (!mail->ctl.done || it0 + k < mail->ctl.iters - 1) tally_pair(1 + k);
            if (sweepErr) break;
            if (mail->ctl.done) {
                ok = true;
                iterations = mail->ctl.iters;
                break;
            }
            it0 += nit;
        }
        if (!ok) iterations = a.maxIter;
    }
    if (sweepErr) {
        cudaMemsetAsync(sw.err, 0, sizeof(int), s);
        cudaMemsetAsync(sw.xchg, 0, sweep_exchange_words(c.I, c.J, c.K) * sizeof(unsigned long long), s);
        cudaMemsetAsync(sw.ticket, 0, 3 * sizeof(unsigned int), s);
        sw.epoch = 0;
        sync();
        if (errMsg) *errMsg = "a wavefront (factor or sweep) gave up waiting for a neighbouring tile";
        return FLIP_E_DEVICE_TIMEOUT;
    }
    res->iterations = iterations;
    res->residual = resid;
    const bool accept = ok || (iterations == a.maxIter && resid < a.accTol);   // pressuresolver.cpp:810-840
    { FLIP_COUNT(1); k_x_to_float<<<nb, TPB, 0, s>>>(n, pb.x, pb.pressure); }
    if (a.dumpPressure) {
        PCK(sync());
        PCK(cudaMemcpy(a.dumpPressure, pb.pressure, n * sizeof(float), cudaMemcpyDeviceToHost));
    }
    if (!accept) return FLIP_E_SOLVER_NOCONV;
    long long tot = (long long)(c.I + 1) * c.J * c.K + (long long)c.I * (c.J + 1) * c.K + (long long)c.I * c.J * (c.K + 1);
    float factor = (float)(a.dt / c.dx);
    { FLIP_COUNT(1); k_apply_pressure<<<div_up(tot, TPB), TPB, 0, s>>>(c, a.phi, a.wu, a.wv, a.ww, pb.pressure, factor,
                                                                    a.u, a.v, a.w, a.vu, a.vv, a.vw); }
    res->applied = true;
    return FLIP_OK;
}

}  // namespace flip
