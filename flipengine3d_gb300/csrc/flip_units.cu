// The MIC(0) preconditioner on its own, through the C ABI: the factor
// (factorModifiedIncompleteColesky0, pcgsolver.h:70-185) and the two
// triangular sweeps (solveLower / solveLowerTransposeInPlace,
// pcgsolver.h:192-221) that the pressure solve runs, on rows the caller
// gives, so that each can be checked against the reference's own routines
// on arbitrary 7-point matrices.  The same kernels and launch sequence as
// inside a solve; only the data comes from host arrays in flat cell order.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/flip3d.h"
#include "flip_device.cuh"

namespace flip {
int record_error(int code, const std::string &msg);   // sets flip_last_error()
}

using namespace flip;

namespace {

// Device buffers of one call, freed on every exit path.
struct Scratch {
    std::vector<void *> ptrs;
    ~Scratch() {
        for (void *p : ptrs) cudaFree(p);
    }
    template <class T>
    bool get(T **p, size_t count) {
        if (cudaMalloc((void **)p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return false;
        ptrs.push_back((void *)*p);
        return true;
    }
};

int cuda_status(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return FLIP_OK;
    return record_error(FLIP_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// The rows must form a system the pressure solve could build: flagged cells
// interior (1..n-2 on every axis) and couplings only between flagged cells.
int check_system(int I, int J, int K, const uint8_t *fluid) {
    if (I < 3 || J < 3 || K < 3) return record_error(FLIP_E_DOMAIN, "grid must be at least 3 cells on each axis");
    if ((long long)I * J * K >= (1LL << 28)) return record_error(FLIP_E_DOMAIN, "grid too large");
    for (int k = 0; k < K; k++)
        for (int j = 0; j < J; j++)
            for (int i = 0; i < I; i++) {
                const bool interior = i >= 1 && j >= 1 && k >= 1 && i <= I - 2 && j <= J - 2 && k <= K - 2;
                if (fluid[i + (size_t)I * (j + (size_t)J * k)] && !interior)
                    return record_error(FLIP_E_DOMAIN, "a flagged cell lies on the grid border");
            }
    return FLIP_OK;
}

StepConsts grid_consts(int I, int J, int K) {
    StepConsts c{};
    c.I = I; c.J = J; c.K = K;
    return c;
}

}  // namespace

extern "C" int flip_mic0_factor(int I, int J, int K, const uint8_t *fluid, const double *rows, double *invdiag) {
    if (!fluid || !rows || !invdiag) return record_error(FLIP_E_NULL, "null pointer");
    int rc = check_system(I, J, K, fluid);
    if (rc) return rc;
    const size_t n = (size_t)I * J * K;
    int lo = 0x7fffffff, hi = -1;
    for (int k = 0; k < K; k++)
        for (int j = 0; j < J; j++)
            for (int i = 0; i < I; i++)
                if (fluid[i + (size_t)I * (j + (size_t)J * k)]) {
                    lo = std::min(lo, i + j + k);
                    hi = std::max(hi, i + j + k);
                }
    std::memset(invdiag, 0, n * sizeof(double));
    if (hi < lo) return FLIP_OK;
    Scratch sc;
    uint8_t *dFluid;
    double4_32a *dAd;
    double *dInv, *dW;
    int *dProgress, *dErr;
    unsigned int *dTicket;
    const int ntiles = mic0_factor_tiles(J, K);
    if (!sc.get(&dFluid, n) || !sc.get(&dAd, n) || !sc.get(&dInv, n) || !sc.get(&dW, 3 * n) ||
        !sc.get(&dProgress, ntiles) || !sc.get(&dErr, 1) || !sc.get(&dTicket, 1))
        return record_error(FLIP_E_NOMEM, "cudaMalloc failed");
    cudaStream_t s = nullptr;
    if ((rc = cuda_status(cudaMemcpy(dFluid, fluid, n, cudaMemcpyHostToDevice), "copy flags")) ||
        (rc = cuda_status(cudaMemcpy(dAd, rows, n * sizeof(double4_32a), cudaMemcpyHostToDevice), "copy rows")) ||
        (rc = cuda_status(cudaMemset(dInv, 0, n * sizeof(double)), "clear")) ||
        (rc = cuda_status(cudaMemset(dErr, 0, sizeof(int)), "clear")))
        return rc;
    mic0_factor(grid_consts(I, J, K), dFluid, dAd, dInv, dW, dW + n, dW + 2 * n, dProgress, dTicket, dErr,
                DEFAULT_SPIN_LIMIT, lo, hi, s);
    if ((rc = cuda_status(cudaDeviceSynchronize(), "factor"))) return rc;
    int err = 0;
    if ((rc = cuda_status(cudaMemcpy(&err, dErr, sizeof(int), cudaMemcpyDeviceToHost), "read flag"))) return rc;
    if (err) return record_error(FLIP_E_DEVICE_TIMEOUT, "the factor's wavefront gave up waiting");
    return cuda_status(cudaMemcpy(invdiag, dInv, n * sizeof(double), cudaMemcpyDeviceToHost), "read pivots");
}

extern "C" int flip_mic0_precondition(int I, int J, int K, const uint8_t *fluid, const float *factor, const float *r,
                                      float *z, int orientation) {
    if (!fluid || !factor || !r || !z) return record_error(FLIP_E_NULL, "null pointer");
    if (orientation < 0 || orientation > 1) return record_error(FLIP_E_OUT_OF_RANGE, "orientation must be 0 or 1");
    int rc = check_system(I, J, K, fluid);
    if (rc) return rc;
    const size_t n = (size_t)I * J * K;
    const SweepLayout g = sweep_layout(I, J, K, orientation);
    const long long nsl = sweep_layout_size(I, J, K);
    // the rows and right-hand side of the interior cells into the sweep layout
    std::vector<float4> hL((size_t)nsl, make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<float> hr((size_t)nsl, 0.0f), hz((size_t)nsl, 0.0f);
    for (int k = 1; k <= K - 2; k++)
        for (int j = 1; j <= J - 2; j++)
            for (int i = 1; i <= I - 2; i++) {
                const size_t t = i + (size_t)I * (j + (size_t)J * k);
                const long long e = sweep_index(g, i, j, k);
                if (fluid[t]) hL[e] = make_float4(factor[4 * t], factor[4 * t + 1], factor[4 * t + 2], factor[4 * t + 3]);
                hr[e] = fluid[t] ? r[t] : 0.0f;
            }
    Scratch sc;
    uint8_t *dFluid;
    float4 *dL;
    float *dR, *dZ;
    int *dSkip;
    SweepState sw{};
    const int nt = sweep_tiles_max(I, J, K);
    const long long nw = sweep_exchange_words(I, J, K);
    if (!sc.get(&dFluid, n) || !sc.get(&dL, nsl) || !sc.get(&dR, nsl) || !sc.get(&dZ, nsl) || !sc.get(&dSkip, 1) ||
        !sc.get(&sw.range, nt) || !sc.get(&sw.xchg, nw) || !sc.get(&sw.ticket, 4) || !sc.get(&sw.err, 4))
        return record_error(FLIP_E_NOMEM, "cudaMalloc failed");
    sw.xchgWords = nw;
    if ((rc = cuda_status(cudaMemcpy(dFluid, fluid, n, cudaMemcpyHostToDevice), "copy flags")) ||
        (rc = cuda_status(cudaMemcpy(dL, hL.data(), nsl * sizeof(float4), cudaMemcpyHostToDevice), "copy rows")) ||
        (rc = cuda_status(cudaMemcpy(dR, hr.data(), nsl * sizeof(float), cudaMemcpyHostToDevice), "copy rhs")) ||
        (rc = cuda_status(cudaMemset(dZ, 0, nsl * sizeof(float)), "clear")) ||
        (rc = cuda_status(cudaMemset(dSkip, 0, sizeof(int)), "clear")) ||
        (rc = cuda_status(cudaMemset(sw.xchg, 0, nw * sizeof(unsigned long long)), "clear")) ||
        (rc = cuda_status(cudaMemset(sw.ticket, 0, 4 * sizeof(unsigned int)), "clear")) ||
        (rc = cuda_status(cudaMemset(sw.err, 0, 4 * sizeof(int)), "clear")))
        return rc;
    const StepConsts c = grid_consts(I, J, K);
    cudaStream_t s = nullptr;
    launch_sweep_ranges(c, g, dFluid, sw, s);
    launch_sweeps(c, g, dL, dR, dZ, sw, dSkip, s);
    if ((rc = cuda_status(cudaDeviceSynchronize(), "sweeps"))) return rc;
    int err = 0;
    if ((rc = cuda_status(cudaMemcpy(&err, sw.err, sizeof(int), cudaMemcpyDeviceToHost), "read flag"))) return rc;
    if (err) return record_error(FLIP_E_DEVICE_TIMEOUT, "a sweep tile gave up waiting");
    if ((rc = cuda_status(cudaMemcpy(hz.data(), dZ, nsl * sizeof(float), cudaMemcpyDeviceToHost), "read result")))
        return rc;
    for (size_t t = 0; t < n; t++) z[t] = 0.0f;
    for (int k = 1; k <= K - 2; k++)
        for (int j = 1; j <= J - 2; j++)
            for (int i = 1; i <= I - 2; i++) {
                const size_t t = i + (size_t)I * (j + (size_t)J * k);
                if (fluid[t]) z[t] = hz[sweep_index(g, i, j, k)];
            }
    return FLIP_OK;
}
