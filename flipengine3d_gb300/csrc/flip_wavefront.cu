// MIC(0) triangular sweeps as a pipelined wavefront (sm_103a).
//
// The preconditioner solve of the reference, solveLower followed by
// solveLowerTransposeInPlace (pcgsolver.h:192-221), over the 7-point factor:
//   forward   y_c = inv_c * (r_c - Lz_{c-z} y_{c-z} - Ly_{c-y} y_{c-y} - Lx_{c-x} y_{c-x})
//   backward  z_c = inv_c * (y_c - Lx_c z_{c+x} - Ly_c z_{c+y} - Lz_c z_{c+z})
// with the subtractions in the reference's column order and FP32 rounding
// of every product and difference.  A cell depends on its three lower
// (upper) neighbours only, so the cells of a plane i + j + k = const are
// independent: the exact wavefront order.
//
// Mapping.  A CTA owns a tile of 32 (j) x 8 (k) pencils along i: lane = j,
// warp = k.  In the forward sweep thread (l, w) processes i = 1 + t - l - w
// at step t, so its j-1 neighbour (lane l-1) and k-1 neighbour (warp w-1)
// finished that i at step t-1: j terms arrive by warp shuffle, k terms
// through shared memory after the per-step barrier (the backward sweep is the
// mirror image).  In the forward sweep a cell hands its neighbours the
// finished products L_c * y_c rather than y_c: each product is rounded once,
// by whichever thread forms it, so the bits are the reference's and the
// receiver saves the coupling load and the multiply.
//
// Lean steps.  A pencil's cells outside the interior (the skewed start and
// end of the wavefront, and pencils past the grid's edge) are read at the
// nearest boundary cell, whose factor row and right-hand side are zero, so
// every step runs the same unpredicated arithmetic and only the store is
// masked.  Steps run in chunks of 8; the next chunk's rows, right-hand side
// and edge words are loaded while the current one computes.
//
// Tile edges.  The lanes on a tile's downstream edges publish each term they
// form as one 64-bit word {sweep epoch, value} in an exchange array; the
// neighbouring tile polls exactly the words it needs until their epoch is the
// current sweep's.  A single naturally aligned 64-bit store is seen whole or
// not at all, so no fence, flag or progress counter sits between the
// producing step and the consuming one.  Cells that the producing tile does
// not compute (outside its range of system cells) contribute zero and are not
// polled.  Tiles take tickets in dependency order, so a tile only waits for
// tiles that are already running.  Every wait is bounded: on timeout the tile
// raises the error flag and stops, and the host reports
// FLIP_E_DEVICE_TIMEOUT; no wait can spin forever.
#include "flip_device.cuh"

namespace flip {

namespace {

constexpr int TJ = 32, TK = 8, CH = 8;
constexpr int NTHREADS = TJ * TK;
constexpr unsigned int SPIN_LIMIT = 1u << 22;   // poll rounds of <= ~250 ns: about a second

struct SweepArgs {
    const float4 *L;
    const float *rin;              // forward: r rounded to FP32; backward: unused (reads out)
    float *out;                    // forward: y; backward: z, in place over y
    int I, J, K;
    int ntj, ntk;
    const int2 *range;             // per tile: first/last step (forward numbering) holding a system cell
    unsigned long long *xchg;      // per tile: TK j-edge rows, then TJ k-edge rows, of I words
    unsigned int *ticket;
    unsigned int ticketBase;
    unsigned int epoch;
    int *err;
};

__device__ __forceinline__ unsigned long long ld_word(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_word(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long pack(unsigned int epoch, float v) {
    return ((unsigned long long)epoch << 32) | __float_as_uint(v);
}
__device__ __forceinline__ float word_value(unsigned long long v) { return __uint_as_float((unsigned int)v); }

template <bool FWD>
__global__ void __launch_bounds__(NTHREADS, 1) k_wavefront(SweepArgs a) {
    // forward: L_w * y of each pencil's last cell (the k+1 neighbour's term);
    // backward: z of each pencil's last cell
    __shared__ float shP[2][TK][TJ];
    __shared__ int shTile;
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int ntiles = a.ntj * a.ntk;
    if (threadIdx.x == 0) {
        int t = (int)(atomicAdd(a.ticket, 1u) - a.ticketBase);
        shTile = FWD ? t : ntiles - 1 - t;
    }
    __syncthreads();
    const int tile = shTile;
    if (tile < 0 || tile >= ntiles) return;
    const int tj = tile % a.ntj, tk = tile / a.ntj;
    const int NI = a.I - 2;
    const int T = NI + (TJ - 1) + (TK - 1);
    auto steps_of = [&](int tl) {   // [first, last] step of a tile in this sweep's numbering
        const int2 rg = a.range[tl];
        return FWD ? rg : make_int2((T - 1) - rg.y, (T - 1) - rg.x);
    };
    const int2 own = steps_of(tile);
    const int tlo = own.x, thi = own.y;
    if (thi < tlo) return;   // no system cell in the tile: nothing to compute or publish

    const int j = 1 + tj * TJ + l, k = 1 + tk * TK + w;
    const bool active = j <= a.J - 2 && k <= a.K - 2;
    const long long row = (long long)a.I * (min(j, a.J - 1) + (long long)a.J * min(k, a.K - 1));
    const float4 *Lrow = a.L + row;
    const float *Rrow = FWD ? a.rin + row : a.out + row;
    float *Orow = a.out + row;
    // cell of step t: i0 + t (forward) or i0 - t (backward)
    const int i0 = FWD ? 1 - l - w : NI + (TJ - 1 - l) + (TK - 1 - w);
    // steps at which the cell is interior and inside the tile's range
    int v0 = FWD ? l + w : i0 - NI;
    int v1 = v0 + NI - 1;
    if (!active) { v0 = 1; v1 = 0; }
    v0 = max(v0, tlo);
    v1 = min(v1, thi);

    const int srcJ = FWD ? (tj > 0 ? tile - 1 : -1) : (tj < a.ntj - 1 ? tile + 1 : -1);
    const int srcK = FWD ? (tk > 0 ? tile - a.ntj : -1) : (tk < a.ntk - 1 ? tile + a.ntj : -1);
    const bool rdJ = (FWD ? l == 0 : l == TJ - 1) && srcJ >= 0;   // reads the j neighbour tile
    const bool rdK = (FWD ? w == 0 : w == TK - 1) && srcK >= 0;   // reads the k neighbour tile
    const bool pubJ = FWD ? (l == TJ - 1 && tj < a.ntj - 1) : (l == 0 && tj > 0);
    const bool pubK = FWD ? (w == TK - 1 && tk < a.ntk - 1) : (w == 0 && tk > 0);
    const size_t rowsPerTile = (size_t)(TJ + TK) * a.I;
    unsigned long long *pubJrow = a.xchg + tile * rowsPerTile + (size_t)w * a.I;
    unsigned long long *pubKrow = a.xchg + tile * rowsPerTile + (size_t)(TK + l) * a.I;
    const unsigned long long *srcJrow = a.xchg + (rdJ ? srcJ : 0) * rowsPerTile + (size_t)w * a.I;
    const unsigned long long *srcKrow = a.xchg + (rdK ? srcK : 0) * rowsPerTile + (size_t)(TK + l) * a.I;
    // steps whose edge word must come from the neighbour: this cell is
    // computed and the neighbour's cell (TJ-1 or TK-1 steps later there) too
    int nJ0 = 1, nJ1 = 0, nK0 = 1, nK1 = 0;
    if (rdJ) {
        const int2 rg = steps_of(srcJ);
        nJ0 = max(v0, rg.x - (TJ - 1));
        nJ1 = min(v1, rg.y - (TJ - 1));
    }
    if (rdK) {
        const int2 rg = steps_of(srcK);
        nK0 = max(v0, rg.x - (TK - 1));
        nK1 = min(v1, rg.y - (TK - 1));
    }
    const unsigned int ep = a.epoch;

    struct Chunk {
        float4 L[CH];
        float r[CH];
        unsigned long long eJ[CH], eK[CH];
        unsigned int needJ, needK;   // bit s: the edge word of step s comes from the neighbour
    };
    auto cell = [&](int t) { return FWD ? i0 + t : i0 - t; };
    auto load = [&](Chunk &d, int tb) {
        d.needJ = 0;
        d.needK = 0;
#pragma unroll
        for (int s = 0; s < CH; s++) {
            const int t = tb + s;
            const int i = cell(t);
            const int ic = min(max(i, 0), a.I - 1);
            d.L[s] = __ldg(Lrow + ic);
            d.r[s] = __ldg(Rrow + ic);
            const bool nj = t >= nJ0 && t <= nJ1, nk = t >= nK0 && t <= nK1;
            d.eJ[s] = nj ? ld_word(srcJrow + i) : 0ull;
            d.eK[s] = nk ? ld_word(srcKrow + i) : 0ull;
            d.needJ |= nj ? 1u << s : 0u;
            d.needK |= nk ? 1u << s : 0u;
        }
    };
    // Re-poll the edge words of the chunk that are not yet of this sweep;
    // false when the wait gave up (or another tile raised the error flag).
    auto settle = [&](Chunk &d, int tb) -> bool {
        if (!(d.needJ | d.needK)) return true;
        unsigned int spin = 0;
        for (;;) {
            unsigned int missJ = 0, missK = 0;
#pragma unroll
            for (int s = 0; s < CH; s++) {
                missJ |= ((d.needJ >> s) & 1u) && (unsigned int)(d.eJ[s] >> 32) != ep ? 1u << s : 0u;
                missK |= ((d.needK >> s) & 1u) && (unsigned int)(d.eK[s] >> 32) != ep ? 1u << s : 0u;
            }
            if (!(missJ | missK)) return true;
            if (++spin > SPIN_LIMIT || *(volatile int *)a.err) return false;
            if (spin > 8) __nanosleep(64);
#pragma unroll
            for (int s = 0; s < CH; s++) {
                const int i = cell(tb + s);
                if ((missJ >> s) & 1u) d.eJ[s] = ld_word(srcJrow + i);
                if ((missK >> s) & 1u) d.eK[s] = ld_word(srcKrow + i);
            }
        }
    };

    shP[0][w][l] = 0.0f;
    shP[1][w][l] = 0.0f;
    // forward: this pencil's terms from its last cell, L_x y (own next cell)
    // and L_y y (lane l+1); backward: z of its last cell
    float px = 0.0f, pz = 0.0f, zPrev = 0.0f;
    auto run = [&](Chunk &cur, Chunk &nxt, int tb) -> bool {
        const bool fine = settle(cur, tb);
        if (__syncthreads_or(!fine)) {
            if (!fine) atomicExch(a.err, 1);
            return false;
        }
        if (tb + CH <= thi) load(nxt, tb + CH);
        const int par = tb & 1;
#pragma unroll
        for (int s = 0; s < CH; s++) {
            const int t = tb + s;
            const int cb = (s & 1) ^ par, pb = cb ^ 1;   // buffers of steps t and t-1
            const float4 Lc = cur.L[s];
            float res;
            if (FWD) {
                float pJ = __shfl_up_sync(0xffffffffu, pz, 1);
                if (l == 0) pJ = word_value(cur.eJ[s]);
                const float pK = w > 0 ? shP[pb][w - 1][l] : word_value(cur.eK[s]);
                float acc = __fsub_rn(cur.r[s], pK);
                acc = __fsub_rn(acc, pJ);
                acc = __fsub_rn(acc, px);
                res = __fmul_rn(acc, Lc.x);
                px = __fmul_rn(Lc.y, res);
                pz = __fmul_rn(Lc.z, res);
                const float pw = __fmul_rn(Lc.w, res);
                shP[cb][w][l] = pw;
                const bool valid = t >= v0 && t <= v1;
                const int i = cell(t);
                if (valid) Orow[i] = res;
                if (valid && pubJ) st_word(pubJrow + i, pack(ep, pz));
                if (valid && pubK) st_word(pubKrow + i, pack(ep, pw));
            } else {
                float zJ = __shfl_down_sync(0xffffffffu, zPrev, 1);
                if (l == TJ - 1) zJ = word_value(cur.eJ[s]);
                const float zK = w < TK - 1 ? shP[pb][w + 1][l] : word_value(cur.eK[s]);
                float acc = __fsub_rn(cur.r[s], __fmul_rn(Lc.y, zPrev));
                acc = __fsub_rn(acc, __fmul_rn(Lc.z, zJ));
                acc = __fsub_rn(acc, __fmul_rn(Lc.w, zK));
                res = __fmul_rn(acc, Lc.x);
                zPrev = res;
                shP[cb][w][l] = res;
                const bool valid = t >= v0 && t <= v1;
                const int i = cell(t);
                if (valid) Orow[i] = res;
                if (valid && pubJ) st_word(pubJrow + i, pack(ep, res));
                if (valid && pubK) st_word(pubKrow + i, pack(ep, res));
            }
            if (t == thi) break;
            __syncthreads();
        }
        return true;
    };

    Chunk A, B;
    load(A, tlo);
    for (int tb = tlo; tb <= thi; tb += 2 * CH) {
        if (!run(A, B, tb)) return;
        if (tb + CH > thi) break;
        if (!run(B, A, tb + CH)) return;
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
long long sweep_exchange_words(int I, int J, int K) {
    int ntj, ntk;
    return (long long)sweep_tiles(J, K, &ntj, &ntk) * (TJ + TK) * I;
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

void launch_sweeps(const StepConsts &c, const float4 *L, const float *rf, float *z, SweepState &sw, cudaStream_t s) {
    int ntj, ntk;
    int n = sweep_tiles(c.J, c.K, &ntj, &ntk);
    if (sw.epoch >= 0xfffffff0u) {   // epochs are about to wrap: forget every old word
        cudaMemsetAsync(sw.xchg, 0, sweep_exchange_words(c.I, c.J, c.K) * sizeof(unsigned long long), s);
        sw.epoch = 0;
    }
    SweepArgs a;
    a.L = L; a.rin = rf; a.out = z;
    a.I = c.I; a.J = c.J; a.K = c.K;
    a.ntj = ntj; a.ntk = ntk;
    a.range = sw.range; a.xchg = sw.xchg; a.ticket = sw.ticket; a.err = sw.err;
    a.epoch = ++sw.epoch;
    a.ticketBase = (unsigned int)(sw.launches * n);
    sw.launches++;
    { FLIP_COUNT(1); k_wavefront<true><<<n, NTHREADS, 0, s>>>(a); }
    a.epoch = ++sw.epoch;
    a.ticketBase = (unsigned int)(sw.launches * n);
    sw.launches++;
    { FLIP_COUNT(1); k_wavefront<false><<<n, NTHREADS, 0, s>>>(a); }
}

}  // namespace flip
