// MIC(0) triangular sweeps as a pipelined wavefront (sm_103a).
//
// The preconditioner solve of the reference, solveLower followed by
// solveLowerTransposeInPlace (pcgsolver.h:192-221), over the 7-point factor:
//   forward   y_c = inv_c * (r_c - Lz_{c-z} y_{c-z} - Ly_{c-y} y_{c-y} - Lx_{c-x} y_{c-x})
//   backward  z_c = inv_c * (y_c - Lx_c z_{c+x} - Ly_c z_{c+y} - Lz_c z_{c+z})
// with the subtractions in the reference's column order.  A cell depends on
// its three lower (upper) neighbours only, so the cells of a plane
// i + j + k = const are independent: the exact wavefront order.
//
// Mapping: a CTA owns a tile of 32 (j) x 8 (k) pencils along i; lane = j,
// warp = k.  In the forward sweep thread (l, w) processes i = 1 + t - l - w
// at step t, so its j-1 neighbour (lane l-1) and k-1 neighbour (warp w-1)
// finished that i at step t-1: j values arrive by warp shuffle, k values
// through shared memory after the per-step barrier (the backward sweep is the
// mirror image).  Tiles exchange their edge pencils through global memory:
// each tile publishes its progress (steps done) after every chunk of steps;
// a consumer checks it once per chunk and then loads the chunk's edge values
// together.  Tiles take tickets in dependency order, so a tile only waits for
// tiles that are already running.  Every wait is bounded: on timeout the tile
// raises the error flag and stops, and the host reports
// FLIP_E_DEVICE_TIMEOUT; no wait can spin forever.
#include "flip_kernels.cuh"

namespace flip {

namespace {

constexpr int TJ = 32, TK = 8, CHUNK = 8;
constexpr unsigned int SPIN_LIMIT = 1u << 22;   // polls of ~256 ns each: about a second

struct SweepArgs {
    const float4 *L;
    const double *rin;       // forward: r (FP64, rounded to FP32 on load); backward: unused
    float *out;              // forward: y; backward: z, in place over y
    int I, J, K;
    int ntj, ntk;
    const int2 *range;       // per tile: first/last step (forward numbering) holding a system cell
    unsigned int *progress;  // per tile: epoch << 20 | steps done
    unsigned int *ticket;
    unsigned int ticketBase;
    unsigned int epoch;
    int *err;
};

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned int *p, unsigned int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned int tag(unsigned int epoch, int steps) {
    return ((epoch & 0xfffu) << 20) | (unsigned int)steps;
}

// Wait until `tile` has done `need` steps of this sweep; false on abort.
__device__ bool wait_progress(const SweepArgs &a, int tile, int need) {
    const unsigned int ep = a.epoch & 0xfffu;
    for (unsigned int spin = 0; spin < SPIN_LIMIT; spin++) {
        unsigned int v = ld_acquire(&a.progress[tile]);
        if ((v >> 20) == ep && (int)(v & 0xfffffu) >= need) return true;
        if (*(volatile int *)a.err) return false;
        __nanosleep(256);
    }
    atomicExch(a.err, 1);
    return false;
}

template <bool FWD>
__global__ void __launch_bounds__(TJ *TK) k_sweep(SweepArgs a) {
    __shared__ float shY[2][TK][TJ];   // value of each pencil at the last step
    __shared__ float shL[2][TK][TJ];   // forward: its coupling to the next k cell (L.w)
    __shared__ int shTile, shAbort;
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int ntiles = a.ntj * a.ntk;
    if (threadIdx.x == 0) {
        int t = (int)(atomicAdd(a.ticket, 1u) - a.ticketBase);
        shTile = FWD ? t : ntiles - 1 - t;
        shAbort = 0;
    }
    __syncthreads();
    const int tile = shTile;
    if (tile < 0 || tile >= ntiles) return;
    const int tj = tile % a.ntj, tk = tile / a.ntj;
    const long long sy = a.I, sz = (long long)a.I * a.J;
    const int j = 1 + tj * TJ + l, k = 1 + tk * TK + w;
    const bool active = j <= a.J - 2 && k <= a.K - 2;
    const int NI = a.I - 2;
    const int T = NI + (TJ - 1) + (TK - 1);
    const int2 rg = a.range[tile];
    const int tlo = FWD ? rg.x : (T - 1) - rg.y;
    const int thi = FWD ? rg.y : (T - 1) - rg.x;
    const int srcJ = FWD ? (tj > 0 ? tile - 1 : -1) : (tj < a.ntj - 1 ? tile + 1 : -1);
    const int srcK = FWD ? (tk > 0 ? tile - a.ntj : -1) : (tk < a.ntk - 1 ? tile + a.ntj : -1);
    const bool edgeJ = FWD ? (l == 0) : (l == TJ - 1);
    const bool edgeK = FWD ? (w == 0) : (w == TK - 1);

    if (thi < tlo) {   // no system cell in the tile: every value of it is zero
        if (threadIdx.x == 0) st_release(&a.progress[tile], tag(a.epoch, T));
        return;
    }
    // the lower (upper) neighbour of a pencil's first cell is outside the
    // system: start from zeros
    shY[0][w][l] = 0.0f;
    shY[1][w][l] = 0.0f;
    shL[0][w][l] = 0.0f;
    shL[1][w][l] = 0.0f;
    __syncthreads();
    if (threadIdx.x == 0) st_release(&a.progress[tile], tag(a.epoch, tlo));

    float yPrev = 0.0f;    // this pencil's value at its previous cell
    float LxPrev = 0.0f;   // forward: coupling of the previous cell to this one (L.y)
    float LzPass = 0.0f;   // forward: coupling of this pencil's last cell to the next lane (L.z)
    for (int tb = tlo; tb <= thi; tb += CHUNK) {
        // own data of the chunk (independent of the other tiles)
        float4 Lr[CHUNK];
        float rr[CHUNK], LJr[CHUNK], LKr[CHUNK], bJ[CHUNK], bK[CHUNK];
        long long cs[CHUNK];
        bool oks[CHUNK];
#pragma unroll
        for (int s = 0; s < CHUNK; s++) {
            int t = tb + s;
            int i = FWD ? 1 + t - l - w : NI - (t - (TJ - 1 - l) - (TK - 1 - w));
            bool ok = active && i >= 1 && i <= NI && t <= thi;
            long long c = (long long)i + sy * j + sz * k;
            oks[s] = ok;
            cs[s] = c;
            Lr[s] = ok ? a.L[c] : make_float4(0.f, 0.f, 0.f, 0.f);
            rr[s] = ok ? (FWD ? (float)a.rin[c] : a.out[c]) : 0.0f;
            LJr[s] = (FWD && ok && edgeJ && srcJ >= 0) ? a.L[c - sy].z : 0.0f;
            LKr[s] = (FWD && ok && edgeK && srcK >= 0) ? a.L[c - sz].w : 0.0f;
        }
        // the producers must cover this chunk's edge cells
        if (threadIdx.x == 0) {
            int hi = min(tb + CHUNK - 1, thi);
            bool go = true;
            if (srcJ >= 0) go = wait_progress(a, srcJ, min(hi + TJ + 1, T));
            if (go && srcK >= 0) go = wait_progress(a, srcK, min(hi + TK + 1, T));
            if (!go) shAbort = 1;
        }
        __syncthreads();
        if (shAbort) return;
#pragma unroll
        for (int s = 0; s < CHUNK; s++) {
            long long c = cs[s];
            bJ[s] = (oks[s] && edgeJ && srcJ >= 0) ? __ldcg(&a.out[FWD ? c - sy : c + sy]) : 0.0f;
            bK[s] = (oks[s] && edgeK && srcK >= 0) ? __ldcg(&a.out[FWD ? c - sz : c + sz]) : 0.0f;
        }
#pragma unroll
        for (int s = 0; s < CHUNK; s++) {
            const int t = tb + s;
            const bool ok = oks[s];
            const float4 Lc = Lr[s];
            float res = 0.0f;
            if (FWD) {
                float yJ = __shfl_up_sync(0xffffffffu, yPrev, 1);
                float LJ = __shfl_up_sync(0xffffffffu, LzPass, 1);
                float yK = 0.0f, LK = 0.0f;
                if (w > 0) { yK = shY[(t - 1) & 1][w - 1][l]; LK = shL[(t - 1) & 1][w - 1][l]; }
                else { yK = bK[s]; LK = LKr[s]; }
                if (l == 0) { yJ = bJ[s]; LJ = LJr[s]; }
                if (ok) {
                    float acc = rr[s];
                    acc = __fsub_rn(acc, __fmul_rn(LK, yK));
                    acc = __fsub_rn(acc, __fmul_rn(LJ, yJ));
                    acc = __fsub_rn(acc, __fmul_rn(LxPrev, yPrev));
                    res = __fmul_rn(acc, Lc.x);
                    a.out[cs[s]] = res;
                }
                shY[t & 1][w][l] = res;
                shL[t & 1][w][l] = Lc.w;
                yPrev = res;
                LxPrev = Lc.y;
                LzPass = Lc.z;
            } else {
                float zJ = __shfl_down_sync(0xffffffffu, yPrev, 1);
                float zK = (w < TK - 1) ? shY[(t - 1) & 1][w + 1][l] : bK[s];
                if (l == TJ - 1) zJ = bJ[s];
                if (ok) {
                    float acc = rr[s];
                    acc = __fsub_rn(acc, __fmul_rn(Lc.y, yPrev));
                    acc = __fsub_rn(acc, __fmul_rn(Lc.z, zJ));
                    acc = __fsub_rn(acc, __fmul_rn(Lc.w, zK));
                    res = __fmul_rn(acc, Lc.x);
                    a.out[cs[s]] = res;
                }
                shY[t & 1][w][l] = res;
                yPrev = res;
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            __threadfence();
            int done = tb + CHUNK > thi ? T : tb + CHUNK;
            st_release(&a.progress[tile], tag(a.epoch, done));
        }
    }
}

__global__ void k_tile_range_init(int2 *range, int n) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) range[t] = make_int2(0x7fffffff, -1);
}

// First and last forward step at which a tile meets a system cell
// (lanes of a warp that fall into the same tile reduce before the atomics).
__global__ void k_tile_range(const uint8_t *fluid, int I, int J, int K, int ntj, int2 *range) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool f = t < (long long)I * J * K && fluid[t];
    int tile = -1, step = 0;
    if (f) {
        int i = (int)(t % I), j = (int)((t / I) % J), k = (int)(t / ((long long)I * J));
        tile = (j - 1) / TJ + ntj * ((k - 1) / TK);
        step = (i - 1) + (j - 1) % TJ + (k - 1) % TK;
    }
    unsigned int grp = __match_any_sync(0xffffffffu, tile);
    int mn = __reduce_min_sync(grp, f ? step : 0x7fffffff);
    int mx = __reduce_max_sync(grp, f ? step : -1);
    if (f && (int)(threadIdx.x & 31) == __ffs(grp) - 1) {
        atomicMin(&range[tile].x, mn);
        atomicMax(&range[tile].y, mx);
    }
}

}  // namespace

int sweep_tiles(int J, int K, int *ntj, int *ntk) {
    *ntj = (J - 2 + TJ - 1) / TJ;
    *ntk = (K - 2 + TK - 1) / TK;
    return *ntj * *ntk;
}

void launch_sweep_ranges(const StepConsts &c, const uint8_t *fluid, SweepState &sw, cudaStream_t s) {
    int ntj, ntk;
    int n = sweep_tiles(c.J, c.K, &ntj, &ntk);
    { FLIP_COUNT(1); k_tile_range_init<<<div_up(n, 256), 256, 0, s>>>(sw.range, n); }
    long long nc = (long long)c.I * c.J * c.K;
    { FLIP_COUNT(1); k_tile_range<<<div_up(nc, 256), 256, 0, s>>>(fluid, c.I, c.J, c.K, ntj, sw.range); }
    cudaMemsetAsync(sw.ticket, 0, sizeof(unsigned int), s);
    sw.launches = 0;
}

void launch_sweeps(const StepConsts &c, const float4 *L, const double *r, float *z, SweepState &sw, cudaStream_t s) {
    int ntj, ntk;
    int n = sweep_tiles(c.J, c.K, &ntj, &ntk);
    SweepArgs a;
    a.L = L; a.rin = r; a.out = z;
    a.I = c.I; a.J = c.J; a.K = c.K;
    a.ntj = ntj; a.ntk = ntk;
    a.range = sw.range; a.progress = sw.progress; a.ticket = sw.ticket; a.err = sw.err;
    a.epoch = ++sw.epoch;
    a.ticketBase = (unsigned int)(sw.launches * n);
    sw.launches++;
    { FLIP_COUNT(1); k_sweep<true><<<n, TJ * TK, 0, s>>>(a); }
    a.epoch = ++sw.epoch;
    a.ticketBase = (unsigned int)(sw.launches * n);
    sw.launches++;
    { FLIP_COUNT(1); k_sweep<false><<<n, TJ * TK, 0, s>>>(a); }
}

}  // namespace flip
