// Variational pressure projection for GB300 (sm_103a).
//
// The system is the reference's (pressuresolver.cpp:580-808): a 7-point
// matrix over interior cells with phi < 0, ghost-fluid diagonal terms at
// air neighbours, face weights from the solid level set.  It is never
// assembled: rows are rebuilt from phi and the face weights where needed.
// Preconditioner: the reference's MIC(0) (pcgsolver.h:70-185, tau 0.97,
// pivot floor 0.25) restated for 7-point rows; its factorisation and the two
// triangular sweeps run as i+j+k wavefronts, so the preconditioner is the
// reference's own.  Precision: factorisation, RHS, the solution vector, dot
// products and a true-residual recompute every 25 iterations are FP64; the
// Laplacian apply, the sweeps and the vector updates are FP32.
#include "flip_kernels.cuh"

namespace flip {

namespace {

constexpr int TPB = 256;

struct RowD {
    double diag, xm, xp, ym, yp, zm, zp;
};

__device__ __forceinline__ bool sys_cell(const StepConsts &c, const float *phi, int i, int j, int k) {
    if (i < 1 || j < 1 || k < 1 || i > c.I - 2 || j > c.J - 2 || k > c.K - 2) return false;
    return phi[(long long)i + (long long)c.I * ((long long)j + (long long)c.J * k)] < 0.0f;
}

// One matrix row in FP64, as _calculateMatrixCoefficientsThread builds it
// (pressuresolver.cpp:723-808).  Off-diagonal entries exist only towards
// neighbours that are rows of the system; a liquid neighbour outside the
// interior contributes neither an entry nor a ghost-fluid term (the
// reference's key map drops it).
__device__ RowD row_coeffs(const StepConsts &c, const float *phi, const float *wu, const float *wv,
                           const float *ww, double mf, int i, int j, int k) {
    Dims du{c.I + 1, c.J, c.K}, dv{c.I, c.J + 1, c.K}, dw{c.I, c.J, c.K + 1}, dc{c.I, c.J, c.K};
    double vR = wu[du.idx(i + 1, j, k)], vL = wu[du.idx(i, j, k)];
    double vT = wv[dv.idx(i, j + 1, k)], vB = wv[dv.idx(i, j, k)];
    double vF = ww[dw.idx(i, j, k + 1)], vK = ww[dw.idx(i, j, k)];
    double pc = phi[dc.idx(i, j, k)];
    RowD r;
    r.diag = (vR + vL + vT + vB + vF + vK) * mf;
    r.xm = r.xp = r.ym = r.yp = r.zm = r.zp = 0.0;
    const double maxtheta = 25.0, eps = 1e-9;
    const int nb[6][3] = {{i + 1, j, k}, {i - 1, j, k}, {i, j + 1, k}, {i, j - 1, k}, {i, j, k + 1}, {i, j, k - 1}};
    const double vol[6] = {vR, vL, vT, vB, vF, vK};
    double *off[6] = {&r.xp, &r.xm, &r.yp, &r.ym, &r.zp, &r.zm};
#pragma unroll
    for (int q = 0; q < 6; q++) {
        double pn = phi[dc.idx(nb[q][0], nb[q][1], nb[q][2])];
        if (pn < 0.0) {
            if (sys_cell(c, phi, nb[q][0], nb[q][1], nb[q][2])) *off[q] = -vol[q] * mf;
        } else {
            double theta = pn / (pc + eps);
            theta = fmax(-maxtheta, fmin(theta, maxtheta));
            r.diag -= vol[q] * mf * theta;
        }
    }
    r.diag = fmax(r.diag, 0.0);
    return r;
}

__global__ void k_flags(StepConsts c, const float *phi, uint8_t *fluid, int *levelRange) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    Dims d{c.I, c.J, c.K};
    if (t >= d.size()) return;
    int i = (int)(t % c.I), j = (int)((t / c.I) % c.J), k = (int)(t / ((long long)c.I * c.J));
    bool f = sys_cell(c, phi, i, j, k);
    fluid[t] = f ? 1 : 0;
    if (f) {
        atomicMin(&levelRange[0], i + j + k);
        atomicMax(&levelRange[1], i + j + k);
        atomicAdd(&levelRange[2], 1);
    }
}

// RHS (pressuresolver.cpp:580-669, zero solid velocities) and FP32 copies of
// the matrix rows.
__global__ void k_build(StepConsts c, const float *phi, const uint8_t *fluid, const float *wu, const float *wv,
                        const float *ww, const float *u, const float *v, const float *w, double mf,
                        PressureBuffers pb, unsigned long long *bmaxBits) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    Dims d{c.I, c.J, c.K};
    if (t >= d.size()) return;
    pb.x[t] = 0.0;
    pb.r[t] = 0.0f;
    pb.z[t] = 0.0f;
    pb.s[t] = 0.0f;
    pb.q[t] = 0.0f;
    if (!fluid[t]) {
        pb.A[t] = make_float4(0.f, 0.f, 0.f, 0.f);
        pb.Adiag[t] = 0.0;
        pb.b[t] = 0.0;
        pb.invdiagD[t] = 0.0;
        pb.L[t] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    int i = (int)(t % c.I), j = (int)((t / c.I) % c.J), k = (int)(t / ((long long)c.I * c.J));
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
    atomicMax(bmaxBits, (unsigned long long)__double_as_longlong(fabs(div)));
    RowD r = row_coeffs(c, phi, wu, wv, ww, mf, i, j, k);
    pb.Adiag[t] = r.diag;
    pb.A[t] = make_float4((float)r.diag, (float)r.xp, (float)r.yp, (float)r.zp);
}

// MIC(0) pivots for one wavefront i+j+k = level, in FP64.  The column
// oriented elimination of factorModifiedIncompleteColesky0 reduces, for
// 7-point rows, to: d_c = A_cc - sum over earlier neighbours k (ascending) of
//   L_ck^2 + 0.97 * L_ck * (sum of k's other later-neighbour entries L_mk),
// L_mk = A_mk / sqrt(pivot_k); a pivot below 0.25*A_kk falls back to A_kk.
__global__ void k_mic0_level(StepConsts c, const uint8_t *fluid, const float *wu, const float *wv, const float *ww,
                             double mf, const double *Adiag, double *invD, int level) {
    int jj = blockIdx.x * blockDim.x + threadIdx.x;
    int nj = c.J - 2, nk = c.K - 2;
    if (jj >= nj * nk) return;
    int j = 1 + jj % nj, k = 1 + jj / nj;
    int i = level - j - k;
    if (i < 1 || i > c.I - 2) return;
    Dims dc{c.I, c.J, c.K}, du{c.I + 1, c.J, c.K}, dv{c.I, c.J + 1, c.K}, dw{c.I, c.J, c.K + 1};
    long long t = dc.idx(i, j, k);
    if (!fluid[t]) return;
    double ad = Adiag[t];
    double d = ad;
    // earlier neighbours in ascending index order: -z, -y, -x
    const int nb[3][3] = {{i, j, k - 1}, {i, j - 1, k}, {i - 1, j, k}};
    for (int q = 0; q < 3; q++) {
        int a = nb[q][0], b = nb[q][1], e = nb[q][2];
        long long kk = dc.idx(a, b, e);
        if (!fluid[kk] || Adiag[kk] == 0.0) continue;
        double inv = invD[kk];
        double wck = q == 0 ? ww[dw.idx(i, j, k)] : (q == 1 ? wv[dv.idx(i, j, k)] : wu[du.idx(i, j, k)]);
        double Lck = (-wck * mf) * inv;
        // k's later neighbours, ascending: +x, +y, +z; c itself excluded
        double miss = 0.0;
        if (q != 2 && fluid[dc.idx(a + 1, b, e)]) miss += (-(double)wu[du.idx(a + 1, b, e)] * mf) * inv;
        if (q != 1 && fluid[dc.idx(a, b + 1, e)]) miss += (-(double)wv[dv.idx(a, b + 1, e)] * mf) * inv;
        if (q != 0 && fluid[dc.idx(a, b, e + 1)]) miss += (-(double)ww[dw.idx(a, b, e + 1)] * mf) * inv;
        d -= Lck * Lck;
        d -= 0.97 * Lck * miss;
    }
    double inv;
    if (ad == 0.0) inv = 0.0;
    else if (d < 0.25 * ad) inv = 1 / sqrt(ad);
    else inv = 1 / sqrt(d);
    invD[t] = inv;
}

__global__ void k_mic0_finalize(StepConsts c, const uint8_t *fluid, const float *wu, const float *wv,
                                const float *ww, double mf, const double *invD, float4 *L) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    Dims dc{c.I, c.J, c.K}, du{c.I + 1, c.J, c.K}, dv{c.I, c.J + 1, c.K}, dw{c.I, c.J, c.K + 1};
    if (t >= dc.size()) return;
    if (!fluid[t] || invD[t] == 0.0) { L[t] = make_float4(0.f, 0.f, 0.f, 0.f); return; }
    int i = (int)(t % c.I), j = (int)((t / c.I) % c.J), k = (int)(t / ((long long)c.I * c.J));
    double inv = invD[t];
    float lx = fluid[dc.idx(i + 1, j, k)] ? (float)((-(double)wu[du.idx(i + 1, j, k)] * mf) * inv) : 0.0f;
    float ly = fluid[dc.idx(i, j + 1, k)] ? (float)((-(double)wv[dv.idx(i, j + 1, k)] * mf) * inv) : 0.0f;
    float lz = fluid[dc.idx(i, j, k + 1)] ? (float)((-(double)ww[dw.idx(i, j, k + 1)] * mf) * inv) : 0.0f;
    L[t] = make_float4((float)inv, lx, ly, lz);
}

// Forward sweep L y = r for one wavefront (solveLower, pcgsolver.h:192-205).
__global__ void k_fwd_level(StepConsts c, const uint8_t *fluid, const float4 *L, const float *r, float *y, int level) {
    int jj = blockIdx.x * blockDim.x + threadIdx.x;
    int nj = c.J - 2, nk = c.K - 2;
    if (jj >= nj * nk) return;
    int j = 1 + jj % nj, k = 1 + jj / nj;
    int i = level - j - k;
    if (i < 1 || i > c.I - 2) return;
    long long sy = c.I, sz = (long long)c.I * c.J;
    long long t = i + sy * j + sz * k;
    if (!fluid[t]) return;
    float acc = r[t];
    acc = __fsub_rn(acc, __fmul_rn(L[t - sz].w, y[t - sz]));
    acc = __fsub_rn(acc, __fmul_rn(L[t - sy].z, y[t - sy]));
    acc = __fsub_rn(acc, __fmul_rn(L[t - 1].y, y[t - 1]));
    y[t] = __fmul_rn(acc, L[t].x);
}

// Backward sweep L^T z = y for one wavefront (solveLowerTransposeInPlace,
// pcgsolver.h:208-221), in place over y.
__global__ void k_bwd_level(StepConsts c, const uint8_t *fluid, const float4 *L, float *z, int level) {
    int jj = blockIdx.x * blockDim.x + threadIdx.x;
    int nj = c.J - 2, nk = c.K - 2;
    if (jj >= nj * nk) return;
    int j = 1 + jj % nj, k = 1 + jj / nj;
    int i = level - j - k;
    if (i < 1 || i > c.I - 2) return;
    long long sy = c.I, sz = (long long)c.I * c.J;
    long long t = i + sy * j + sz * k;
    if (!fluid[t]) return;
    float4 l = L[t];
    float acc = z[t];
    acc = __fsub_rn(acc, __fmul_rn(l.y, z[t + 1]));
    acc = __fsub_rn(acc, __fmul_rn(l.z, z[t + sy]));
    acc = __fsub_rn(acc, __fmul_rn(l.w, z[t + sz]));
    z[t] = __fmul_rn(acc, l.x);
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) s += sh[q];
    __syncthreads();
    return s;
}

// q = A s (FP32 stencil), block partials of s.q in FP64
__global__ void k_spmv(StepConsts c, const uint8_t *fluid, const float4 *A, const float *s, float *q,
                       double *partials) {
    __shared__ double sh[32];
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n = (long long)c.I * c.J * c.K;
    double part = 0.0;
    if (t < n && fluid[t]) {
        long long sy = c.I, sz = (long long)c.I * c.J;
        float4 a = A[t];
        float acc = __fmul_rn(a.x, s[t]);
        acc = __fmaf_rn(a.y, s[t + 1], acc);
        acc = __fmaf_rn(a.z, s[t + sy], acc);
        acc = __fmaf_rn(a.w, s[t + sz], acc);
        acc = __fmaf_rn(A[t - 1].y, s[t - 1], acc);
        acc = __fmaf_rn(A[t - sy].z, s[t - sy], acc);
        acc = __fmaf_rn(A[t - sz].w, s[t - sz], acc);
        q[t] = acc;
        part = (double)s[t] * (double)acc;
    }
    double b = block_sum(part, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = b;
}

__global__ void k_dot(long long n, const float *a, const float *b, double *partials) {
    __shared__ double sh[32];
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double part = t < n ? (double)a[t] * (double)b[t] : 0.0;
    double s = block_sum(part, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// fixed-order final sum of the block partials (deterministic)
__global__ void k_sum_partials(const double *partials, int n, double *out) {
    __shared__ double sh[32];
    double v = 0.0;
    for (int q = threadIdx.x; q < n; q += blockDim.x) v += partials[q];
    double s = block_sum(v, sh);
    if (threadIdx.x == 0) *out = s;
}

__device__ __forceinline__ void block_max_to(float v, unsigned int *out) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && v > 0.0f) atomicMax(out, __float_as_uint(v));
}

// x += alpha s (FP64), r -= alpha q (FP32), |r|inf (BLAS::addScaled with a
// float alpha, blaswrapper.h:129-158)
__global__ void k_update_xr(long long n, const uint8_t *fluid, double *x, float *r, const float *s, const float *q,
                            const double *scal, unsigned int *rmaxBits) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const float alpha = (float)(scal[3] / scal[0]);   // alpha = rho / (s.q), passed on as float
    float m = 0.0f;
    if (t < n && fluid[t]) {
        x[t] += (double)alpha * (double)s[t];
        float rv = __fmaf_rn(-alpha, q[t], r[t]);
        r[t] = rv;
        m = fabsf(rv);
    }
    block_max_to(m, rmaxBits);
}

// r = b - A x in FP64 with the rows rebuilt in FP64 (residual replacement)
__global__ void k_true_residual(StepConsts c, const float *phi, const uint8_t *fluid, const float *wu,
                                const float *wv, const float *ww, double mf, const double *b, const double *x,
                                float *r, unsigned int *rmaxBits) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n = (long long)c.I * c.J * c.K;
    float m = 0.0f;
    if (t < n && fluid[t]) {
        int i = (int)(t % c.I), j = (int)((t / c.I) % c.J), k = (int)(t / ((long long)c.I * c.J));
        long long sy = c.I, sz = (long long)c.I * c.J;
        RowD row = row_coeffs(c, phi, wu, wv, ww, mf, i, j, k);
        double ax = row.diag * x[t] + row.xp * x[t + 1] + row.xm * x[t - 1] + row.yp * x[t + sy] +
                    row.ym * x[t - sy] + row.zp * x[t + sz] + row.zm * x[t - sz];
        float rv = (float)(b[t] - ax);
        r[t] = rv;
        m = fabsf(rv);
    }
    block_max_to(m, rmaxBits);
}

__global__ void k_update_s(long long n, const uint8_t *fluid, const float *z, float *s, const double *scal) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const float beta = (float)(scal[1] / scal[3]);    // beta = rho_new / rho
    if (t < n && fluid[t]) s[t] = __fmaf_rn(beta, s[t], z[t]);
}

__global__ void k_set_rho(double *scal) { scal[3] = scal[1]; }

__global__ void k_init_rs(long long n, const double *b, float *r, unsigned int *rmaxBits) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    float m = 0.0f;
    if (t < n) {
        float rv = (float)b[t];
        r[t] = rv;
        m = fabsf(rv);
    }
    block_max_to(m, rmaxBits);
}

__global__ void k_copy_float(long long n, const float *a, float *b) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) b[t] = a[t];
}

__global__ void k_x_to_float(long long n, const double *x, float *p) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) p[t] = (float)x[t];
}

// _applyPressureToVelocityFieldThread (pressuresolver.cpp:896-1046), without
// surface tension.  Liquid here means phi < 0 over all cells
// (FluidMaterialGrid, :849-858); the faces i == 0 and i == I-1 (and the v/w
// analogues) are skipped as the reference skips them.
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
    int i = (int)(l % ni), j = (int)((l / ni) % nj), k = (int)(l / ((long long)ni * nj));
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

}  // namespace

int pressure_partials(const StepConsts &c) { return (int)div_up((long long)c.I * c.J * c.K, TPB); }

void launch_pressure_build(const StepConsts &c, const float *phi, const float *wu, const float *wv,
                           const float *ww, const float *u, const float *v, const float *w, double dt,
                           PressureBuffers &pb, cudaStream_t s) {
    long long n = (long long)c.I * c.J * c.K;
    int lr[3] = {0x7fffffff, -1, 0};
    cudaMemcpyAsync(pb.levelRange, lr, sizeof(lr), cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(pb.scal, 0, 4 * sizeof(double), s);
    { FLIP_COUNT(1); k_flags<<<div_up(n, TPB), TPB, 0, s>>>(c, phi, pb.fluid, pb.levelRange); }
    double mf = dt / (c.dx * c.dx);
    FLIP_COUNT(1);
    k_build<<<div_up(n, TPB), TPB, 0, s>>>(c, phi, pb.fluid, wu, wv, ww, u, v, w, mf, pb,
                                           (unsigned long long *)(pb.scal + 2));
}

void launch_mic0_factor(const StepConsts &c, const float *phi, const float *wu, const float *wv, const float *ww,
                        double dt, PressureBuffers &pb, int levelLo, int levelHi, cudaStream_t s) {
    (void)phi;
    double mf = dt / (c.dx * c.dx);
    int np = (c.J - 2) * (c.K - 2);
    for (int l = levelLo; l <= levelHi; l++)
        { FLIP_COUNT(1); k_mic0_level<<<div_up(np, TPB), TPB, 0, s>>>(c, pb.fluid, wu, wv, ww, mf, pb.Adiag, pb.invdiagD, l); }
    long long n = (long long)c.I * c.J * c.K;
    { FLIP_COUNT(1); k_mic0_finalize<<<div_up(n, TPB), TPB, 0, s>>>(c, pb.fluid, wu, wv, ww, mf, pb.invdiagD, pb.L); }
}

void launch_precondition(const StepConsts &c, PressureBuffers &pb, const float *rin, float *zout, int levelLo,
                         int levelHi, cudaStream_t s) {
    int np = (c.J - 2) * (c.K - 2);
    for (int l = levelLo; l <= levelHi; l++)
        { FLIP_COUNT(1); k_fwd_level<<<div_up(np, TPB), TPB, 0, s>>>(c, pb.fluid, pb.L, rin, zout, l); }
    for (int l = levelHi; l >= levelLo; l--)
        { FLIP_COUNT(1); k_bwd_level<<<div_up(np, TPB), TPB, 0, s>>>(c, pb.fluid, pb.L, zout, l); }
}

void launch_spmv_dot(const StepConsts &c, PressureBuffers &pb, cudaStream_t s) {
    long long n = (long long)c.I * c.J * c.K;
    { FLIP_COUNT(1); k_spmv<<<div_up(n, TPB), TPB, 0, s>>>(c, pb.fluid, pb.A, pb.s, pb.q, pb.partials); }
    { FLIP_COUNT(1); k_sum_partials<<<1, 1024, 0, s>>>(pb.partials, pb.nPartials, pb.scal + 0); }
}

void launch_dot_zr(const StepConsts &c, PressureBuffers &pb, cudaStream_t s) {
    long long n = (long long)c.I * c.J * c.K;
    { FLIP_COUNT(1); k_dot<<<div_up(n, TPB), TPB, 0, s>>>(n, pb.z, pb.r, pb.partials); }
    { FLIP_COUNT(1); k_sum_partials<<<1, 1024, 0, s>>>(pb.partials, pb.nPartials, pb.scal + 1); }
}

void launch_update_xr(const StepConsts &c, PressureBuffers &pb, cudaStream_t s) {
    long long n = (long long)c.I * c.J * c.K;
    cudaMemsetAsync(pb.rmaxBits, 0, sizeof(unsigned int), s);
    { FLIP_COUNT(1); k_update_xr<<<div_up(n, TPB), TPB, 0, s>>>(n, pb.fluid, pb.x, pb.r, pb.s, pb.q, pb.scal, pb.rmaxBits); }
}

void launch_init_residual(const StepConsts &c, PressureBuffers &pb, cudaStream_t s) {
    long long n = (long long)c.I * c.J * c.K;
    cudaMemsetAsync(pb.rmaxBits, 0, sizeof(unsigned int), s);
    { FLIP_COUNT(1); k_init_rs<<<div_up(n, TPB), TPB, 0, s>>>(n, pb.b, pb.r, pb.rmaxBits); }
}

void launch_set_rho(PressureBuffers &pb, cudaStream_t s) {
    { FLIP_COUNT(1); k_set_rho<<<1, 1, 0, s>>>(pb.scal); }
}

void launch_copy_zs(const StepConsts &c, PressureBuffers &pb, cudaStream_t s) {
    long long n = (long long)c.I * c.J * c.K;
    { FLIP_COUNT(1); k_copy_float<<<div_up(n, TPB), TPB, 0, s>>>(n, pb.z, pb.s); }
}

void launch_copy_qr(const StepConsts &c, PressureBuffers &pb, cudaStream_t s) {
    long long n = (long long)c.I * c.J * c.K;
    { FLIP_COUNT(1); k_copy_float<<<div_up(n, TPB), TPB, 0, s>>>(n, pb.q, pb.r); }
}

void launch_true_residual(const StepConsts &c, const float *phi, const float *wu, const float *wv,
                          const float *ww, double dt, PressureBuffers &pb, float *out, unsigned int *rmaxOut,
                          cudaStream_t s) {
    long long n = (long long)c.I * c.J * c.K;
    double mf = dt / (c.dx * c.dx);
    cudaMemsetAsync(rmaxOut, 0, sizeof(unsigned int), s);
    { FLIP_COUNT(1); k_true_residual<<<div_up(n, TPB), TPB, 0, s>>>(c, phi, pb.fluid, wu, wv, ww, mf, pb.b, pb.x, out, rmaxOut); }
}

void launch_update_s(const StepConsts &c, PressureBuffers &pb, cudaStream_t s) {
    long long n = (long long)c.I * c.J * c.K;
    { FLIP_COUNT(1); k_update_s<<<div_up(n, TPB), TPB, 0, s>>>(n, pb.fluid, pb.z, pb.s, pb.scal); }
}

void launch_pressure_to_float(const StepConsts &c, PressureBuffers &pb, cudaStream_t s) {
    long long n = (long long)c.I * c.J * c.K;
    { FLIP_COUNT(1); k_x_to_float<<<div_up(n, TPB), TPB, 0, s>>>(n, pb.x, pb.pressure); }
}

void launch_apply_pressure(const StepConsts &c, const float *phi, const float *wu, const float *wv,
                           const float *ww, const PressureBuffers &pb, double dt, float *u, float *v, float *w,
                           uint8_t *vu, uint8_t *vv, uint8_t *vw, cudaStream_t s) {
    long long tot = (long long)(c.I + 1) * c.J * c.K + (long long)c.I * (c.J + 1) * c.K +
                    (long long)c.I * c.J * (c.K + 1);
    float factor = (float)(dt / c.dx);
    { FLIP_COUNT(1); k_apply_pressure<<<div_up(tot, TPB), TPB, 0, s>>>(c, phi, wu, wv, ww, pb.pressure, factor, u, v, w, vu, vv, vw); }
}

}  // namespace flip
