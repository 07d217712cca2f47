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
// Mapping.  A CTA owns a tile of 32 (j) x 8 (k) pencils along i: lane l
// of the tile holds the 8 pencils (l, w) of its column, the tile's "slots"
// w = 0..7, and four compute warps take two slots each.  In the forward
// sweep slot w of lane l processes i = 1 + t - l - w at step t, so a cell's
// three lower neighbours (i-1 in the same slot, j-1 in lane l-1, k-1 in
// slot w-1) were all formed at step t - 1: the j terms arrive by warp
// shuffle, the i terms and the k terms between a warp's own slots stay in
// registers, and the k term that crosses to the next warp goes through
// shared memory around the one barrier per step of the compute warps (the
// backward sweep is the mirror image).  A full chunk of steps runs as
// straight-line code, with no test or vote between its steps.  In the
// forward sweep a cell hands its neighbours the finished products L_c * y_c
// rather than y_c: each product is rounded once, by whichever thread forms
// it, so the bits are the reference's.
//
// Data movement.  The factor rows and the right-hand side live in the
// step-major sweep layout (flip_device.cuh), so the 8 steps of a chunk of a
// tile are one contiguous block in either direction.  A loader warp moves
// whole chunks with bulk asynchronous copies into a ring of five
// shared-memory slots as soon as a slot is free (an mbarrier per slot counts
// the bytes in) and prefetches the chunk one ring further ahead into L2; an
// edge warp fetches the terms that the neighbouring tiles publish for the
// chunk's edge cells.  The two run independently, so a tile waiting for its
// neighbours still has its operands on the way.  The compute warps read
// the next step's operands from the slot while they compute the current
// one and store each result straight to global memory (128 contiguous bytes
// per slot and step); cells outside the grid read zero rows, so a step is
// unpredicated.
//
// Where a step's time goes (one warp, measured): the arithmetic and
// shuffles of 8 slots take about 80 cycles, of 2 slots about 46; operands
// from shared memory, result stores and a test or vote per step (which
// splits the unrolled chunk into separate blocks) add 100-250 cycles at 8
// slots.  Four warps of two slots each, in lockstep, with full chunks free
// of tests, sweep the 128^3 dam region in 53 us per launch and a fully
// liquid 128^3 box in 95 us (eight warps of one slot with tests per step:
// 64 us and 95 us; the same in lockstep without tests: 55 us and 82 us).
//
// Tile edges.  The threads on a tile's downstream edges publish each term
// they form as one 64-bit word {sweep epoch, value}, indexed by step, in an
// exchange array; the neighbour's edge warp polls exactly the words its
// chunk needs until their epoch is the current sweep's.  A single naturally
// aligned 64-bit store is seen whole or not at all, so no fence, flag or
// progress counter sits between the producing step and the consuming one.
// Cells that the producing tile does not compute contribute zero and are not
// polled.  Tiles take tickets in dependency order, so a tile only waits for
// tiles that are already running.  Every wait is bounded: on timeout the
// tile raises the error flag and stops, and the host reports
// FLIP_E_DEVICE_TIMEOUT; no wait can spin forever.
#include <atomic>

#include "flip_device.cuh"

namespace flip {

namespace {

#ifndef SWEEP_CH
#define SWEEP_CH 8   // steps per chunk
#endif
constexpr int TJ = SWEEP_TJ, TK = SWEEP_TK, NP = SWEEP_NP, CH = SWEEP_CH, SL = SWEEP_SL, SW = SWEEP_SW;
// one compute warp holds a tile's TK pencils of each lane in registers: a
// cell's three lower neighbours are then all one step back
static_assert(SL == 1 && SW == 1 && CH >= 1, "the compute warp expects skews of one step");
#ifndef SWEEP_NBUF
#define SWEEP_NBUF 5   // ring slots that fit in shared memory
#endif
constexpr int NBUF = SWEEP_NBUF;
static_assert(NBUF >= 2, "the ring needs a slot in flight beside the one in use");
// the edge warp's lanes take the CH x TK j-edge words JQ at a time and the
// CH x TJ k-edge words one step each
constexpr int JQ = CH * TK / 32;
static_assert((CH * TK) % 32 == 0 && TJ == 32 && JQ <= 32, "edge-word mapping of the edge warp");
#ifndef SWEEP_SPW
#define SWEEP_SPW 2   // slots (pencils along the warp axis) per compute warp
#endif
constexpr int SPW = SWEEP_SPW, NWC = TK / SPW;   // compute warps per tile
static_assert(TK % SPW == 0, "a compute warp holds whole slots");
constexpr int NCOMP = 32 * NWC, LOADER = NWC, EDGE = LOADER + 1, NTHREADS = NCOMP + 64;
// Waiting for this CTA's own bulk copies in flight (they complete by
// themselves) keeps the default limit, whatever limit the edge waits have.
constexpr unsigned int DRAIN_SPIN_LIMIT = DEFAULT_SPIN_LIMIT;

struct SweepArgs {
    const float4 *L;               // factor rows, sweep layout
    const float *rin;              // right-hand side, sweep layout (backward: the forward result)
    float *out;                    // result, sweep layout (backward: in place over the forward result)
    int J, K, NI, T;               // J, K: grid extents along the tile's lane and slot axes
    int ntj, ntk;
    const int2 *range;             // per tile: first/last step (forward numbering) holding a system cell
    unsigned long long *xchg;      // per tile: T x TK j-edge words, then T x TJ k-edge words
    unsigned int *ticket;          // [0] forward tile tickets, [1] the pair's epoch, [2] backward tile tickets
                                   // (set by sweep_prep before each pair)
    int *err;
    const int *skip;   // nonzero: return at once
    unsigned int spinLimit;    // poll rounds before a wait gives up
    unsigned int epochSkew;    // 0; nonzero only to make the edge waits run out (fault injection)
};

struct Slot {
    float4 L[CH][NP];   // rows in layout order: forward row q = step q, backward row q = step CH-1-q
    float r[CH][NP];
    float eJ[CH][TK];   // by step: term from the neighbour tile along the lanes, for the edge lane of each slot
    float eK[CH][TJ];   // by step: term from the neighbour tile along the slots, for each lane of the edge slot
};
struct SweepSmem {
    Slot slot[NBUF];
    // per slot: operand bytes in (the loader), edge terms in (the edge warp),
    // chunk done (the compute warps)
    unsigned long long loaded[NBUF], edges[NBUF], done[NBUF];
    // between compute warps g and g + 1, by step parity and lane: forward
    // warp g's last slot's L_z y, backward warp g + 1's first slot's z
    float hand[2][NWC > 1 ? NWC - 1 : 1][TJ];
    int abort;
    int tile;
    unsigned int epoch;
};
static_assert(sizeof(SweepSmem) <= 227 * 1024, "the sweep's shared memory fits one CTA");

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned long long ld_word(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long pack(unsigned int epoch, float v) {
    return ((unsigned long long)epoch << 32) | __float_as_uint(v);
}
__device__ __forceinline__ void mb_init(unsigned long long *b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mb_arrive(unsigned long long *b) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}" ::"r"(smem_addr(b)) : "memory");
}
__device__ __forceinline__ void mb_arrive_expect_tx(unsigned long long *b, unsigned bytes) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(smem_addr(b)),
                 "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mb_test(unsigned long long *b, unsigned parity) {
    unsigned ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok) : "r"(smem_addr(b)), "r"(parity) : "memory");
    return ok != 0;
}
// One round of waiting for a phase: the thread is suspended until the phase
// completes or about `ns` nanoseconds pass, so waiting warps take no issue
// slots from the warps that compute on the same scheduler.
__device__ __forceinline__ bool mb_try(unsigned long long *b, unsigned parity, unsigned ns) {
    unsigned ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok) : "r"(smem_addr(b)), "r"(parity), "r"(ns) : "memory");
    return ok != 0;
}
// Bounded wait for a phase of an mbarrier; false on abort or timeout (which
// raises the abort and error flags).
__device__ bool mb_wait(unsigned long long *b, unsigned parity, int *abortFlag, int *err, unsigned int limit) {
    for (unsigned int spin = 0; spin < limit; spin++) {
        if (mb_try(b, parity, 256)) return true;
        if (*(volatile int *)abortFlag) return false;
    }
    *(volatile int *)abortFlag = 1;
    atomicExch(err, 1);
    return false;
}
// bulk copy global -> shared, completion counted in bytes on mbarrier b
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, unsigned long long *b) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(b)) : "memory");
}
__device__ __forceinline__ void prefetch_l2(const void *src, unsigned bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}
// named barrier of the compute warps, plain and with an OR vote
__device__ __forceinline__ bool compute_sync_or(bool v) {
    unsigned r;
    asm volatile("{\n .reg .pred pi, po;\n setp.ne.u32 pi, %1, 0;\n bar.red.or.pred po, 1, %2, pi;\n selp.u32 %0, 1, 0, po;\n}"
                 : "=r"(r) : "r"((unsigned)v), "n"(NCOMP) : "memory");
    return r != 0;
}
__device__ __forceinline__ void compute_sync() { asm volatile("bar.sync 1, %0;" ::"n"(NCOMP) : "memory"); }
// A published edge term, stored where `on` holds: a predicated store, not a
// branch around one (only the tile's edge lanes publish), ordered against
// nothing else (a consumer reads the word alone), so the compiler may move
// the loads of later steps above it.
__device__ __forceinline__ void st_term(bool on, unsigned long long *p, unsigned long long v) {
    asm volatile("{\n .reg .pred q;\n setp.ne.u32 q, %2, 0;\n @q st.relaxed.gpu.global.u64 [%0], %1;\n}"
                 ::"l"(p), "l"(v), "r"((unsigned)on));
}
// The j-edge terms of a lane's SPW slots at one step: consecutive words.
template <int N>
__device__ __forceinline__ void st_terms(bool on, unsigned long long *p, const float (&v)[N], unsigned int epoch) {
#pragma unroll
    for (int j = 0; j < N; j++) st_term(on, p + j, ((unsigned long long)epoch << 32) | __float_as_uint(v[j]));
}

// SWAP: the tile's lanes run along k and its warps along j (else lanes along
// j, warps along k).  The couplings that travel along each axis and the
// order of the subtractions follow: forward -z, -y, -x; backward +x, +y, +z.
template <bool FWD, bool SWAP>
__global__ void __launch_bounds__(NTHREADS, 1) k_wavefront(SweepArgs a) {
    extern __shared__ __align__(128) unsigned char smemRaw[];
    SweepSmem &sm = *reinterpret_cast<SweepSmem *>(smemRaw);
    const int ntiles = a.ntj * a.ntk;
    if (threadIdx.x == 0) {
        if (*(volatile const int *)a.skip || *(volatile int *)a.err) {
            sm.tile = -1;   // converged, or an earlier sweep gave up: nothing to do
        } else {
            int t = (int)atomicAdd(&a.ticket[FWD ? 0 : 2], 1u);
            sm.tile = FWD ? t : ntiles - 1 - t;
        }
        sm.abort = 0;
        sm.epoch = *(volatile unsigned int *)&a.ticket[1] + (FWD ? 0u : 1u);   // forward e, backward e + 1
        for (int b = 0; b < NBUF; b++) {
            mb_init(&sm.loaded[b], 1);      // the loader's arrival, plus the bytes of the chunk
            mb_init(&sm.edges[b], 32);      // the edge warp's lanes
            mb_init(&sm.done[b], NCOMP);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const int tile = sm.tile;
    if (tile < 0 || tile >= ntiles) return;
    const int tj = tile % a.ntj, tk = tile / a.ntj;
    const int NI = a.NI, T = a.T;
    auto steps_of = [&](int tl) {   // [first, last] step of a tile in this sweep's numbering
        const int2 rg = a.range[tl];
        return FWD ? rg : make_int2((T - 1) - rg.y, (T - 1) - rg.x);
    };
    const int2 own = steps_of(tile);
    const int tlo = own.x, thi = own.y;
    if (thi < tlo) return;   // no system cell in the tile: nothing to compute or publish
    const int nChunks = (thi - tlo) / CH + 1;
    const int j0 = 1 + tj * TJ, k0 = 1 + tk * TK;
    auto pencil_in = [&](int lr, int ww) { return j0 + lr <= a.J - 2 && k0 + ww <= a.K - 2; };
    const size_t wordsPerTile = (size_t)T * (TJ + TK);
    const unsigned int ep = sm.epoch;          // published with this sweep's terms
    const unsigned int epWait = ep + a.epochSkew;   // awaited in the neighbours' words
    // the chunk of steps [tb, tb + rows) as one block of the layout
    auto chunk_rows = [&](int n) { return min(CH, thi + 1 - (tlo + n * CH)); };
    auto chunk_row0 = [&](int rows) { return FWD ? 0 : CH - rows; };
    auto chunk_tf0 = [&](int tb, int rows) { return FWD ? tb : T - tb - rows; };
    const size_t tileBase = (size_t)tile * T * NP;
    const int warp = threadIdx.x >> 5;

    if (warp == LOADER) {
        // ================================================== loader warp
        const int lane = threadIdx.x & 31;
        if (lane != 0) return;
        auto issue = [&](int m, int b) {   // operands of chunk m into slot b
            Slot &sl = sm.slot[b];
            const int tb = tlo + m * CH, rows = chunk_rows(m);
            const unsigned bl = (unsigned)(rows * NP * sizeof(float4)), br = (unsigned)(rows * NP * sizeof(float));
            const size_t e0 = tileBase + (size_t)chunk_tf0(tb, rows) * NP;
            const int r0 = chunk_row0(rows);
            mb_arrive_expect_tx(&sm.loaded[b], bl + br);
            bulk_load(&sl.L[r0][0], a.L + e0, bl, &sm.loaded[b]);
            bulk_load(&sl.r[r0][0], a.rin + e0, br, &sm.loaded[b]);
        };
        auto prefetch = [&](int m) {   // chunk m into L2, for its copy one ring later
            if (m >= nChunks) return;
            const int tb = tlo + m * CH, rows = chunk_rows(m);
            const size_t e0 = tileBase + (size_t)chunk_tf0(tb, rows) * NP;
            prefetch_l2(a.L + e0, (unsigned)(rows * NP * sizeof(float4)));
            prefetch_l2(a.rin + e0, (unsigned)(rows * NP * sizeof(float)));
        };
        int issued = 0;
        for (; issued < nChunks; issued++) {
            const int b = issued % NBUF;
            if (issued >= NBUF &&
                !mb_wait(&sm.done[b], ((issued - NBUF) / NBUF) & 1, &sm.abort, a.err, a.spinLimit))
                break;
            issue(issued, b);
            prefetch(issued + NBUF);
        }
        // The copies started must land before the CTA's shared memory is
        // released, also when the compute warps stop early: each slot's
        // phase completes once its bytes are in.
        for (int m = max(0, issued - NBUF); m < issued; m++)
            for (unsigned int spin = 0;
                 spin < DRAIN_SPIN_LIMIT && !mb_test(&sm.loaded[m % NBUF], (m / NBUF) & 1); spin++)
                __nanosleep(32);
        return;
    }

    if (warp == EDGE) {
        // ==================================================== edge warp
        const int lane = threadIdx.x & 31;
        const int srcJ = FWD ? (tj > 0 ? tile - 1 : -1) : (tj < a.ntj - 1 ? tile + 1 : -1);
        const int srcK = FWD ? (tk > 0 ? tile - a.ntj : -1) : (tk < a.ntk - 1 ? tile + a.ntj : -1);
        const int2 rgJ = srcJ >= 0 ? steps_of(srcJ) : make_int2(1, 0);
        const int2 rgK = srcK >= 0 ? steps_of(srcK) : make_int2(1, 0);
        const int laneJ = FWD ? 0 : TJ - 1, warpK = FWD ? 0 : TK - 1;
        // Each lane's words: for the k edge, the one of its own lane of the
        // upstream tile's edge warp at each step; for the j edge, JQ (step,
        // warp) pairs of each chunk.  A word is needed at step te when the
        // consumer cell is interior (te in [base, base + NI - 1]) and the
        // producer tile computes its cell (te + skew in the producer's
        // range): a window of steps fixed per lane, computed once.
        auto base_of = [&](int lr, int ww) {
            return FWD ? SL * lr + SW * ww : SL * (TJ - 1 - lr) + SW * (TK - 1 - ww);
        };
        int kLo = 1, kHi = 0;
        if (srcK >= 0 && pencil_in(lane, warpK)) {
            const int bs = base_of(lane, warpK);
            kLo = max(bs, rgK.x - SW * (TK - 1));
            kHi = min(min(bs + NI - 1, rgK.y - SW * (TK - 1)), thi);
        }
        const unsigned long long *pK = a.xchg + (srcK >= 0 ? srcK : 0) * wordsPerTile + (size_t)T * TK +
                                       (size_t)SW * (TK - 1) * TJ + lane;   // + te * TJ
        int jLo[JQ], jHi[JQ], jes[JQ];
        const unsigned long long *pJ[JQ];
#pragma unroll
        for (int q = 0; q < JQ; q++) {
            const int e = lane + 32 * q, es = e / TK, ew = e % TK;
            jes[q] = es;
            jLo[q] = 1;
            jHi[q] = 0;
            if (srcJ >= 0 && pencil_in(laneJ, ew)) {
                const int bs = base_of(laneJ, ew);
                jLo[q] = max(bs, rgJ.x - SL * (TJ - 1));
                jHi[q] = min(min(bs + NI - 1, rgJ.y - SL * (TJ - 1)), thi);
            }
            pJ[q] = a.xchg + (srcJ >= 0 ? srcJ : 0) * wordsPerTile + (size_t)SL * (TJ - 1) * TK + ew;   // + te * TK
        }
        bool mine = kLo <= kHi;
#pragma unroll
        for (int q = 0; q < JQ; q++) mine = mine || jLo[q] <= jHi[q];
        const bool anyEdge = __any_sync(0xffffffffu, mine);
        for (int m = 0; m < nChunks; m++) {
            const int b = m % NBUF;
            Slot &sl = sm.slot[b];
            if (m >= NBUF && !mb_wait(&sm.done[b], ((m - NBUF) / NBUF) & 1, &sm.abort, a.err, a.spinLimit))
                return;   // aborting
            const int tb = tlo + m * CH;
            if (!anyEdge) {   // no upstream tile: the edge terms are zero
                if (m < NBUF) {
#pragma unroll
                    for (int q2 = 0; q2 < CH; q2++) sl.eK[q2][lane] = 0.0f;
#pragma unroll
                    for (int q = 0; q < JQ; q++) sl.eJ[jes[q]][(lane + 32 * q) % TK] = 0.0f;
                }
                __syncwarp();
                mb_arrive(&sm.edges[b]);
                continue;
            }
            float vK[CH], vJ[JQ];
            unsigned long long wK[CH], wJ[JQ];
            unsigned int needK = 0, needJ = 0;
#pragma unroll
            for (int s2 = 0; s2 < CH; s2++) {
                const int te = tb + s2;
                const bool need = te >= kLo && te <= kHi;
                wK[s2] = need ? ld_word(pK + (size_t)te * TJ) : 0ull;
                needK |= need ? 1u << s2 : 0u;
            }
#pragma unroll
            for (int q = 0; q < JQ; q++) {
                const int te = tb + jes[q];
                const bool need = te >= jLo[q] && te <= jHi[q];
                wJ[q] = need ? ld_word(pJ[q] + (size_t)te * TK) : 0ull;
                needJ |= need ? 1u << q : 0u;
            }
            bool ok = true;
            for (unsigned int spin = 0;; spin++) {
                unsigned int missK = 0, missJ = 0;
#pragma unroll
                for (int s2 = 0; s2 < CH; s2++)
                    missK |= ((needK >> s2) & 1u) && (unsigned int)(wK[s2] >> 32) != epWait ? 1u << s2 : 0u;
#pragma unroll
                for (int q = 0; q < JQ; q++)
                    missJ |= ((needJ >> q) & 1u) && (unsigned int)(wJ[q] >> 32) != epWait ? 1u << q : 0u;
                if (!(missK | missJ)) break;
                if (spin >= a.spinLimit) {
                    atomicExch(a.err, 1);
                    ok = false;
                    break;
                }
                if (*(volatile int *)&sm.abort || *(volatile int *)a.err) { ok = false; break; }
                if (spin > 64) __nanosleep(32);
#pragma unroll
                for (int s2 = 0; s2 < CH; s2++)
                    if ((missK >> s2) & 1u) wK[s2] = ld_word(pK + (size_t)(tb + s2) * TJ);
#pragma unroll
                for (int q = 0; q < JQ; q++)
                    if ((missJ >> q) & 1u) wJ[q] = ld_word(pJ[q] + (size_t)(tb + jes[q]) * TK);
            }
            if (!__all_sync(0xffffffffu, ok)) {
                // the compute warps and the loader see the flag in their waits
                *(volatile int *)&sm.abort = 1;
                return;
            }
#pragma unroll
            for (int s2 = 0; s2 < CH; s2++) vK[s2] = __uint_as_float((unsigned int)wK[s2]);
#pragma unroll
            for (int q = 0; q < JQ; q++) vJ[q] = __uint_as_float((unsigned int)wJ[q]);
#pragma unroll
            for (int s2 = 0; s2 < CH; s2++) sl.eK[s2][lane] = vK[s2];
#pragma unroll
            for (int q = 0; q < JQ; q++) sl.eJ[jes[q]][(lane + 32 * q) % TK] = vJ[q];
            __syncwarp();
            mb_arrive(&sm.edges[b]);
        }
        return;
    }

    // ====================================================== compute warps
    // Slot w of lane l is pencil (l, w) of the tile; in the forward sweep it
    // meets cell i = 1 + t - l - w at step t.  The three lower neighbours of
    // a cell (i-1 in the same slot, j-1 in lane l-1, k-1 in slot w-1) were
    // all formed at step t - 1, so the slots of a step are independent: the
    // x term stays in the slot's register, the y term comes from lane l-1 by
    // shuffle, the z term from slot w-1.  Compute warp g holds the SPW slots
    // g*SPW.. of every lane and the warps run in lockstep, one barrier per
    // step: the z term that crosses from warp g-1 to warp g is written to
    // shared memory before the barrier and read after it (the backward sweep
    // is the mirror image, its terms handed from warp g+1 to warp g).  Full
    // chunks run without a test per step; only a tile's last chunk checks
    // for its end.
    const int l = threadIdx.x & 31, g = warp;
    const int w0 = g * SPW;   // first slot of this warp
    const bool takes = FWD ? g > 0 : g < NWC - 1;    // receives the z term from a neighbouring warp
    const bool hands = FWD ? g < NWC - 1 : g > 0;    // hands its edge slot's term on
    const bool slotEdgeIn = FWD ? g == 0 : g == NWC - 1;   // reads the upstream tile's k-edge terms
    constexpr int NB = NWC > 1 ? NWC - 1 : 1;
    const int bIn = min(max(FWD ? g - 1 : g, 0), NB - 1), bOut = min(max(FWD ? g : g - 1, 0), NB - 1);
    const bool pubJ = FWD ? (l == TJ - 1 && tj < a.ntj - 1) : (l == 0 && tj > 0);
    // the tile's k-edge slot (TK-1 forward, 0 backward) publishes for its lane
    const bool pubK = (FWD ? tk < a.ntk - 1 && g == NWC - 1 : tk > 0 && g == 0);
    unsigned long long *pubJw = a.xchg + tile * wordsPerTile + w0;                    // [t][TK]
    unsigned long long *pubKw = a.xchg + tile * wordsPerTile + (size_t)T * TK + l;    // [t][TJ]
    // forward: per slot the L_x y (own next cell), L_y y (lane l+1) and
    // L_z y (slot w+1) terms of its last cell, in the tile's orientation;
    // backward: per slot the z of its last cell, which all three take
    float tx[SPW], tl[SPW], tw[SPW];
#pragma unroll
    for (int j = 0; j < SPW; j++) tx[j] = tl[j] = tw[j] = 0.0f;
    float upNext = 0.0f;   // the neighbouring warp's term for the next step (none before the first)
    for (int n = 0; n < nChunks; n++) {
        const int b = n % NBUF;
        const unsigned par = (n / NBUF) & 1;
        const bool fine = mb_wait(&sm.loaded[b], par, &sm.abort, a.err, a.spinLimit) &&
                          mb_wait(&sm.edges[b], par, &sm.abort, a.err, a.spinLimit);
        if (compute_sync_or(!fine)) {   // every compute warp stops, or none
            *(volatile int *)&sm.abort = 1;
            return;
        }
        const Slot &sl = sm.slot[b];
        const int tb = tlo + n * CH, rows = min(CH, thi + 1 - tb);
        // the results of chunk n: row of step tb + s at out0 + s * ostep
        float *out0 = a.out + tileBase + (size_t)(FWD ? tb : T - 1 - tb) * NP + w0 * TJ + l;
        const long long ostep = FWD ? NP : -NP;
        // operands of the next step, loaded while the current one computes
        float4 Ln[SPW];
        float rn[SPW], ejn[SPW], ekn = 0.0f;
        auto load_step = [&](int s) {
            const int q = FWD ? s : CH - 1 - s;
#pragma unroll
            for (int j = 0; j < SPW; j++) {
                Ln[j] = sl.L[q][(w0 + j) * TJ + l];
                rn[j] = sl.r[q][(w0 + j) * TJ + l];
                ejn[j] = sl.eJ[s][w0 + j];
            }
            if (slotEdgeIn) ekn = sl.eK[s][l];
        };
        auto step = [&](int s, bool more) {
            const int t = tb + s;
            float4 Lc[SPW];
            float rr[SPW], ej[SPW];
#pragma unroll
            for (int j = 0; j < SPW; j++) { Lc[j] = Ln[j]; rr[j] = rn[j]; ej[j] = ejn[j]; }
            const float up = slotEdgeIn ? ekn : upNext;   // the z term of the warp's edge slot
            if (more) load_step(s + 1);
            float nb[SPW];   // the lane neighbour's term of each slot
#pragma unroll
            for (int j = 0; j < SPW; j++) {
                nb[j] = FWD ? __shfl_up_sync(0xffffffffu, tl[j], 1) : __shfl_down_sync(0xffffffffu, tx[j], 1);
                if (l == (FWD ? 0 : TJ - 1)) nb[j] = ej[j];
            }
            float nx[SPW], nl[SPW], nw[SPW], res[SPW];
#pragma unroll
            for (int j = 0; j < SPW; j++) {
                if (FWD) {
                    // terms from the lane and slot neighbours: L of the
                    // neighbour towards this cell times its y
                    const float pL = nb[j];
                    const float pW = j > 0 ? tw[j - 1] : up;
                    float acc = __fsub_rn(rr[j], SWAP ? pL : pW);   // -z
                    acc = __fsub_rn(acc, SWAP ? pW : pL);           // -y
                    acc = __fsub_rn(acc, tx[j]);                    // -x
                    res[j] = __fmul_rn(acc, Lc[j].x);
                    nx[j] = __fmul_rn(Lc[j].y, res[j]);
                    nl[j] = __fmul_rn(SWAP ? Lc[j].w : Lc[j].z, res[j]);   // for the next lane
                    nw[j] = __fmul_rn(SWAP ? Lc[j].z : Lc[j].w, res[j]);   // for the next slot
                } else {
                    const float zL = nb[j];
                    const float zW = j < SPW - 1 ? tx[j + 1] : up;
                    float acc = __fsub_rn(rr[j], __fmul_rn(Lc[j].y, tx[j]));          // +x
                    acc = __fsub_rn(acc, __fmul_rn(Lc[j].z, SWAP ? zW : zL));      // +y
                    acc = __fsub_rn(acc, __fmul_rn(Lc[j].w, SWAP ? zL : zW));      // +z
                    res[j] = __fmul_rn(acc, Lc[j].x);
                    nx[j] = nl[j] = nw[j] = res[j];
                }
            }
            // the edge slot's term for the neighbouring warp, by step parity:
            // it reads it after this step's barrier, before the next one
            if (hands) sm.hand[t & 1][bOut][l] = nw[FWD ? SPW - 1 : 0];
#pragma unroll
            for (int j = 0; j < SPW; j++) __stcg(out0 + s * ostep + j * TJ, res[j]);
            // Edge terms of cells outside the grid are published too: a
            // neighbour only polls the words of cells it needs.
            st_terms(pubJ, pubJw + (size_t)t * TK, nl, ep);
            st_term(pubK, pubKw + (size_t)t * TJ, pack(ep, nw[FWD ? SPW - 1 : 0]));
#pragma unroll
            for (int j = 0; j < SPW; j++) { tx[j] = nx[j]; tl[j] = nl[j]; tw[j] = nw[j]; }
            if (NWC > 1) {
                compute_sync();
                if (takes) upNext = sm.hand[t & 1][bIn][l];
            }
        };
        load_step(0);
        if (rows == CH) {
#pragma unroll
            for (int s = 0; s < CH; s++) step(s, s + 1 < CH);
        } else {
#pragma unroll 1
            for (int s = 0; s < rows; s++) step(s, s + 1 < rows);
        }
        mb_arrive(&sm.done[b]);   // the slot may be refilled
    }
}

// Before a sweep pair without a kernel that prepares it (sweep_prep).
__global__ void k_sweep_prep(unsigned int *ticket) { sweep_prep(ticket); }

__global__ void k_tile_range_init(int2 *range, int n) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) range[t] = make_int2(0x7fffffff, -1);
}

// First and last forward step at which a tile meets a system cell
// (lanes of a warp that fall into the same tile reduce before the atomics).
__global__ void k_tile_range(const uint8_t *fluid, int I, int J, int K, SweepLayout g, int2 *range) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool f = t < (long long)I * J * K && fluid[t];
    int tile = -1, step = 0;
    if (f) {
        int i, j, k;
        unflatten(t, I, J, i, j, k);
        const int aa = (g.swap ? k : j) - 1, bb = (g.swap ? j : k) - 1;
        tile = aa / TJ + g.ntj * (bb / TK);
        step = (i - 1) + SL * (aa % TJ) + SW * (bb % TK);
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

int sweep_tiles_max(int I, int J, int K) {
    int best = 0;
    for (int sw = 0; sw < 2; sw++) {
        const SweepLayout g = sweep_layout(I, J, K, sw);
        best = std::max(best, g.ntj * g.ntk);
    }
    return best;
}

// per tile: TK j-edge words and TJ k-edge words for each of its T steps
long long sweep_exchange_words(int I, int J, int K) {
    const SweepLayout g = sweep_layout(I, J, K);
    return (long long)sweep_tiles_max(I, J, K) * (TJ + TK) * g.T;
}

void launch_sweep_ranges(const StepConsts &c, const SweepLayout &g, const uint8_t *fluid, SweepState &sw,
                         cudaStream_t s) {
    const int n = g.ntj * g.ntk;
    { FLIP_COUNT(1); k_tile_range_init<<<div_up(n, 256), 256, 0, s>>>(sw.range, n); }
    long long nc = (long long)c.I * c.J * c.K;
    { FLIP_COUNT(1); k_tile_range<<<div_up(nc, 256), 256, 0, s>>>(fluid, c.I, c.J, c.K, g, sw.range); }
}

void launch_sweeps(const StepConsts &c, const SweepLayout &g, const float4 *L, const float *rf, float *z,
                   SweepState &sw, const int *skip, cudaStream_t s, bool prepped) {
    const int n = g.ntj * g.ntk;
    static std::atomic<unsigned long long> smemSet{0};   // devices on which the slots' shared memory is opted in
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && !((smemSet.load() >> dev) & 1ull)) {   // idempotent, so a race only repeats it
        cudaFuncSetAttribute(k_wavefront<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SweepSmem));
        cudaFuncSetAttribute(k_wavefront<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SweepSmem));
        cudaFuncSetAttribute(k_wavefront<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SweepSmem));
        cudaFuncSetAttribute(k_wavefront<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SweepSmem));
        smemSet.fetch_or(1ull << dev);
    }
    SweepArgs a;
    a.L = L;
    a.J = g.EA; a.K = g.EB; a.NI = c.I - 2; a.T = g.T;   // extents along the lane and warp axes
    a.ntj = g.ntj; a.ntk = g.ntk;
    a.range = sw.range; a.xchg = sw.xchg; a.ticket = sw.ticket; a.err = sw.err; a.skip = skip;
    a.spinLimit = sw.spinLimit ? sw.spinLimit : DEFAULT_SPIN_LIMIT;
    a.epochSkew = sw.stall ? 1u : 0u;
    // forward: y from r
    a.rin = rf; a.out = z;
    if (!prepped) { FLIP_COUNT(1); k_sweep_prep<<<1, 1, 0, s>>>(sw.ticket); }
    if (g.swap) { FLIP_COUNT(1); k_wavefront<true, true><<<n, NTHREADS, sizeof(SweepSmem), s>>>(a); }
    else { FLIP_COUNT(1); k_wavefront<true, false><<<n, NTHREADS, sizeof(SweepSmem), s>>>(a); }
    // backward: z from y, in place
    a.rin = z; a.out = z;
    if (g.swap) { FLIP_COUNT(1); k_wavefront<false, true><<<n, NTHREADS, sizeof(SweepSmem), s>>>(a); }
    else { FLIP_COUNT(1); k_wavefront<false, false><<<n, NTHREADS, sizeof(SweepSmem), s>>>(a); }
    sw.epoch += 2;
}

// Epochs are 32-bit: before they wrap, forget every old word (outside any
// capture: the host calls this between sweeps).
void sweep_epoch_guard(const StepConsts &c, SweepState &sw, long long upcoming, cudaStream_t s) {
    if ((long long)sw.epoch + upcoming < 0xfffffff0LL) return;
    cudaMemsetAsync(sw.xchg, 0, sweep_exchange_words(c.I, c.J, c.K) * sizeof(unsigned long long), s);
    cudaMemsetAsync(sw.ticket, 0, 3 * sizeof(unsigned int), s);
    sw.epoch = 0;
}

}  // namespace flip
