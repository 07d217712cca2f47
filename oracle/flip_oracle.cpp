// CPU oracle for one FLIP step -- TEST INFRASTRUCTURE ONLY (the checker).
//
// A restatement, in plain C++, of the hot path of the reference engine
// (jklae/FLIPEngine3D, src/engine = FLIP Fluids 1.0.9b).  Every stage keeps
// the reference's arithmetic types and operation order so that, on the same
// inputs and the same reduction partition count, its results equal the
// reference engine's bit for bit.  With more than one thread, the loops
// whose iterations write disjoint outputs (blocks of the level set and of
// P2G, particles, extrapolated cells, matrix rows, vector elements, dot
// product partitions) run on threads, as the reference runs them; the
// triangular sweeps and the factorisation stay sequential.  Each function cites the
// reference file:line it restates.  Compile with -ffp-contract=off so no
// multiply-add is fused on any host (the reference's x86-64 -O2 build fuses
// none).
#include "flip_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace orc {

// ---------------------------------------------------------------- vectors
// vmath::vec3 (src/engine/vmath.h:38-60, vmath.cpp:51-117): float xyz,
// every operation component-wise in float.
struct V3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
    V3() {}
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
};
static inline V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator*(float s, V3 v) { return V3(v.x * s, v.y * s, v.z * s); }
static inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float length(V3 a) { return std::sqrt(dot(a, a)); }
// vmath operator/ (vmath.cpp:100-103): multiply by a float reciprocal
static inline V3 divide(V3 v, float s) {
    float inv = (float)(1.0 / s);
    return V3(v.x * inv, v.y * inv, v.z * inv);
}
static inline V3 normalize(V3 v) { return divide(v, length(v)); }

struct GI { int i, j, k; };

// Grid3d helpers (src/engine/grid3d.h:32-135)
static inline GI posToIdx(double x, double y, double z, double dx) {
    double inv = 1.0 / dx;
    return GI{(int)std::floor(x * inv), (int)std::floor(y * inv), (int)std::floor(z * inv)};
}
static inline GI posToIdx(V3 p, double dx) { return posToIdx(p.x, p.y, p.z, dx); }
static inline V3 idxToPos(int i, int j, int k, double dx) {
    return V3((float)((double)(float)i * dx), (float)((double)(float)j * dx), (float)((double)(float)k * dx));
}
static inline V3 cellCenter(int i, int j, int k, double dx) {
    double hw = 0.5 * dx;
    return V3((float)((double)(float)i * dx + hw), (float)((double)(float)j * dx + hw),
              (float)((double)(float)k * dx + hw));
}
static inline bool inRange(int i, int j, int k, int ni, int nj, int nk) {
    return i >= 0 && j >= 0 && k >= 0 && i < ni && j < nj && k < nk;
}
static inline bool onBorder(int i, int j, int k, int ni, int nj, int nk) {
    return i == 0 || j == 0 || k == 0 || i == ni - 1 || j == nj - 1 || k == nk - 1;
}

template <class T>
struct Grid {
    int ni = 0, nj = 0, nk = 0;
    std::vector<T> a;
    void init(int i, int j, int k, T v) { ni = i; nj = j; nk = k; a.assign((size_t)i * j * k, v); }
    size_t idx(int i, int j, int k) const { return (size_t)i + (size_t)ni * ((size_t)j + (size_t)nj * k); }
    T &operator()(int i, int j, int k) { return a[idx(i, j, k)]; }
    const T &operator()(int i, int j, int k) const { return a[idx(i, j, k)]; }
    bool in(int i, int j, int k) const { return inRange(i, j, k, ni, nj, nk); }
    void fill(T v) { std::fill(a.begin(), a.end(), v); }
};

struct Particle { V3 p, v; };

// ThreadUtils::splitRangeIntoIntervals (src/engine/threadutils.cpp:54-72)
static std::vector<int> splitRange(int b, int e, int n) {
    int size = (int)std::floor((double)(e - b) / (double)n);
    int rem = (e - b) - size * n;
    std::vector<int> out;
    out.push_back(b);
    int cur = b;
    for (int i = 0; i < n; i++) {
        int end = cur + size + (i < rem ? 1 : 0);
        out.push_back(end);
        cur = end;
    }
    return out;
}

// f(begin, end) over [0, n) in nt contiguous ranges, one thread each (the
// caller takes the first); only for loops whose iterations are independent.
template <class F>
static void parallel_ranges(int n, int nt, F f) {
    nt = std::max(1, std::min(nt, n));
    if (nt == 1) {
        if (n > 0) f(0, n);
        return;
    }
    std::vector<int> iv = splitRange(0, n, nt);
    std::vector<std::thread> ts;
    for (int t = 1; t < nt; t++) ts.emplace_back(f, iv[t], iv[t + 1]);
    f(iv[0], iv[1]);
    for (auto &th : ts) th.join();
}

// ------------------------------------------------------ level-set helpers
// LevelsetUtils::fractionInside, two and four corners
// (src/engine/levelsetutils.cpp:39-145)
static float fraction2(float l, float r) {
    if (l < 0 && r < 0) return 1;
    if (l < 0 && r >= 0) return l / (l - r);
    if (l >= 0 && r < 0) return r / (r - l);
    return 0;
}
static void cycle4(float *a) {
    float t = a[0];
    a[0] = a[1]; a[1] = a[2]; a[2] = a[3]; a[3] = t;
}
static float fraction4(float bl, float br, float tl, float tr) {
    int inside = (bl < 0) + (tl < 0) + (br < 0) + (tr < 0);
    float L[4] = {bl, br, tr, tl};
    if (inside == 4) return 1;
    if (inside == 3) {
        while (L[0] < 0) cycle4(L);
        float s0 = 1 - fraction2(L[0], L[3]);
        float s1 = 1 - fraction2(L[0], L[1]);
        return 1.0f - 0.5f * s0 * s1;
    }
    if (inside == 2) {
        while (L[0] >= 0 || !(L[1] < 0 || L[2] < 0)) cycle4(L);
        if (L[1] < 0) {
            float sl = fraction2(L[0], L[3]);
            float sr = fraction2(L[1], L[2]);
            return 0.5f * (sl + sr);
        }
        float mid = 0.25f * (L[0] + L[1] + L[2] + L[3]);
        if (mid < 0) {
            float area = 0;
            float s1 = 1 - fraction2(L[0], L[3]);
            float s3 = 1 - fraction2(L[2], L[3]);
            area += 0.5f * s1 * s3;
            float s2 = 1 - fraction2(L[2], L[1]);
            float s0 = 1 - fraction2(L[0], L[1]);
            area += 0.5f * s0 * s2;
            return 1.0f - area;
        }
        float area = 0;
        float s0 = fraction2(L[0], L[1]);
        float s1 = fraction2(L[0], L[3]);
        area += 0.5f * s0 * s1;
        float s2 = fraction2(L[2], L[1]);
        float s3 = fraction2(L[2], L[3]);
        area += 0.5f * s2 * s3;
        return area;
    }
    if (inside == 1) {
        while (L[0] >= 0) cycle4(L);
        float s0 = fraction2(L[0], L[3]);
        float s1 = fraction2(L[0], L[1]);
        return 0.5f * s0 * s1;
    }
    return 0;
}

// Closest point on a triangle, Eberly's region method, in the mixed
// float/double precision of Collision::findClosestPointOnTriangle
// (src/engine/collision.cpp:161-270).  Only non-degenerate triangles occur
// here (an axis-aligned box mesh).
static double clampd(double v, double lo, double hi) { return std::max(lo, std::min(v, hi)); }
static V3 closestOnTriangle(V3 p0, V3 v0, V3 v1, V3 v2) {
    V3 e0 = v1 - v0, e1 = v2 - v0, pv = v0 - p0;
    double a = dot(e0, e0), b = dot(e0, e1), c = dot(e1, e1), d = dot(e0, pv), e = dot(e1, pv);
    double det = a * c - b * b;
    double s = b * e - c * d;
    double t = b * d - a * e;
    if (s + t < det) {
        if (s < 0.0) {
            if (t < 0.0) {
                if (d < 0.0) { s = clampd(-d / a, 0.0, 1.0); t = 0.0; }
                else { s = 0.0; t = clampd(-e / c, 0.0, 1.0); }
            } else { s = 0.0; t = clampd(-e / c, 0.0, 1.0); }
        } else if (t < 0.0) {
            s = clampd(-d / a, 0.0, 1.0); t = 0.0;
        } else {
            double inv = 1.0 / det;
            s *= inv; t *= inv;
        }
    } else {
        if (s < 0.0) {
            double t0 = b + d, t1 = c + e;
            if (t1 > t0) {
                double num = t1 - t0, den = a - 2 * b + c;
                s = clampd(num / den, 0.0, 1.0); t = 1 - s;
            } else { t = clampd(-e / c, 0.0, 1.0); s = 0.0; }
        } else if (t < 0.0) {
            if (a + d > b + e) {
                double num = c + e - b - d, den = a - 2 * b + c;
                s = clampd(num / den, 0.0, 1.0); t = 1 - s;
            } else { s = clampd(-e / c, 0.0, 1.0); t = 0.0; }
        } else {
            double num = c + e - b - d, den = a - 2 * b + c;
            s = clampd(num / den, 0.0, 1.0); t = 1.0 - s;
        }
    }
    return v0 + (float)s * e0 + (float)t * e1;
}

// ------------------------------------------------------------ MIC(0)-PCG
// A row of the 7-point pressure matrix: columns ascending, diagonal included
// (the reference's SparseMatrix rows, pcgsolver/sparsematrix.h:26-110).
struct Row7 { int col[7]; double val[7]; int nnz; };

// SparseColumnLowerFactor (pcgsolver.h:22-58): inverse diagonal and the
// strictly lower part, column by column.
template <class T>
struct LowerFactor {
    std::vector<T> invdiag;
    std::vector<int> colstart, rowidx;
    std::vector<T> lval;
};

// factorModifiedIncompleteColesky0 (pcgsolver.h:70-185), modification 0.97,
// minimum diagonal ratio 0.25, on the lower triangle, column oriented.
static void mic0_factor(const std::vector<Row7> &A, LowerFactor<double> &F) {
    const int n = (int)A.size();
    std::vector<double> adiag(n, 0.0);
    F.invdiag.assign(n, 0.0);
    F.colstart.assign(n + 1, 0);
    F.rowidx.clear();
    F.lval.clear();
    for (int c = 0; c < n; c++) {
        F.colstart[c] = (int)F.rowidx.size();
        for (int q = 0; q < A[c].nnz; q++) {
            if (A[c].col[q] > c) { F.rowidx.push_back(A[c].col[q]); F.lval.push_back(A[c].val[q]); }
            else if (A[c].col[q] == c) { F.invdiag[c] = adiag[c] = A[c].val[q]; }
        }
    }
    F.colstart[n] = (int)F.rowidx.size();
    std::vector<double> &invdiag = F.invdiag, &lval = F.lval;
    const std::vector<int> &colstart = F.colstart, &rowidx = F.rowidx;
    const double mic = 0.97, minRatio = 0.25;
    auto rowHas = [&](int row, int col) {
        for (int q = 0; q < A[row].nnz; q++) if (A[row].col[q] == col) return true;
        return false;
    };
    for (int k = 0; k < n; k++) {
        if (adiag[k] == 0) continue;
        if (invdiag[k] < minRatio * adiag[k]) invdiag[k] = 1 / std::sqrt(adiag[k]);
        else invdiag[k] = 1 / std::sqrt(invdiag[k]);
        for (int p = colstart[k]; p < colstart[k + 1]; p++) lval[p] *= invdiag[k];
        for (int p = colstart[k]; p < colstart[k + 1]; p++) {
            int j = rowidx[p];
            double mult = lval[p];
            double missing = 0;
            int a = colstart[k];
            while (a < colstart[k + 1] && rowidx[a] < j) {
                if (!rowHas(j, rowidx[a])) missing += lval[a];
                a++;
            }
            if (a < colstart[k + 1] && rowidx[a] == j) invdiag[j] -= mult * lval[a];
            a++;
            int bq = colstart[j];
            while (a < colstart[k + 1] && bq < colstart[j + 1]) {
                if (rowidx[bq] < rowidx[a]) bq++;
                else if (rowidx[bq] == rowidx[a]) { lval[bq] -= mult * lval[a]; a++; bq++; }
                else { missing += lval[a]; a++; }
            }
            while (a < colstart[k + 1]) { missing += lval[a]; a++; }
            invdiag[j] -= mic * mult * missing;
        }
    }
}

// The preconditioner solve: solveLower then solveLowerTransposeInPlace
// (pcgsolver.h:192-221), in the factor's arithmetic type T.
template <class T>
static void mic0_apply(const LowerFactor<T> &F, const std::vector<T> &rhs, std::vector<T> &res) {
    const int n = (int)F.invdiag.size();
    res = rhs;
    for (int i = 0; i < n; i++) {
        res[i] *= F.invdiag[i];
        for (int q = F.colstart[i]; q < F.colstart[i + 1]; q++) res[F.rowidx[q]] -= F.lval[q] * res[i];
    }
    int i = n;
    if (n == 0) return;
    do {
        i--;
        for (int q = F.colstart[i]; q < F.colstart[i + 1]; q++) res[i] -= F.lval[q] * res[F.rowidx[q]];
        res[i] *= F.invdiag[i];
    } while (i != 0);
}

// The system of the unit entry points: rows = the flagged cells in flat
// order; rows7[4c] the diagonal of cell c, rows7[4c+1..3] its couplings to
// the +x, +y, +z neighbours (structural entries wherever that neighbour is
// flagged, mirrored into the neighbour's row).
static void unit_system(int I, int J, int K, const uint8_t *fluid, const double *rows7, std::vector<Row7> &A,
                        std::vector<int> &cellOf, std::vector<int> &rowOf) {
    const size_t nc = (size_t)I * J * K;
    rowOf.assign(nc, -1);
    cellOf.clear();
    for (size_t t = 0; t < nc; t++)
        if (fluid[t]) { rowOf[t] = (int)cellOf.size(); cellOf.push_back((int)t); }
    const int n = (int)cellOf.size();
    A.assign(n, Row7{});
    const long long step[3] = {1, (long long)I, (long long)I * J};
    for (int c = 0; c < n; c++) {
        const long long t = cellOf[c];
        int cols[7]; double vals[7]; int m = 0;
        for (int q = 2; q >= 0; q--) {   // lower neighbours, ascending column: -z, -y, -x
            const long long nb = t - step[q];
            if (nb >= 0 && fluid[nb]) { cols[m] = rowOf[nb]; vals[m] = rows7[4 * nb + 1 + q]; m++; }
        }
        cols[m] = c; vals[m] = rows7[4 * t]; m++;
        for (int q = 0; q < 3; q++) {    // upper neighbours, ascending: +x, +y, +z
            const long long nb = t + step[q];
            if (nb < (long long)nc && fluid[nb]) { cols[m] = rowOf[nb]; vals[m] = rows7[4 * t + 1 + q]; m++; }
        }
        for (int a = 0; a < m; a++) { A[c].col[a] = cols[a]; A[c].val[a] = vals[a]; }
        A[c].nnz = m;
    }
}

// ------------------------------------------------------------- simulation
struct Sim {
    int I, J, K;
    double dx;
    int nthreads = 1;
    double picRatio = 0.05;
    std::vector<V3> bodyForces;
    double cfl = 5.0;
    double tol = 1e-9;
    double accTol = 1.0;
    int maxIter = 1000;
    const int minFrameSteps = 1, maxFrameSteps = 6;
    const float solidBuffer = 0.1f;
    const int maxPerCell = 250;
    const double maxRemovePct = 0.0005;
    const int maxRemoveAbs = 35;
    const float stepFactor = 0.5f;
    const int nearFactor = 3;
    const int exactBand = 3;

    bool initialized = false;
    std::vector<Particle> loadQueue;
    std::vector<Particle> parts;
    int frame = 0, stepNumber = 0;
    double frameDt = 0, frameRemaining = 0, stepDt = 0;
    bool outputInitialized = false;
    int lastSubsteps = 0;

    double sdfRadius = 0;
    Grid<float> solidPhi;          // nodal (I+1)(J+1)(K+1)
    Grid<float> wU, wV, wW;        // face weights
    Grid<uint8_t> nearSolid;
    double nearCell = 0;
    Grid<float> phi;               // liquid SDF, cells
    Grid<float> u, v, w;           // MAC velocity
    Grid<uint8_t> vu, vv, vw;      // valid masks
    Grid<float> su, sv, sw;        // saved field
    int lastIters = 0;
    double lastError = 0;
    bool solidBuilt = false;

    Sim(int i, int j, int k, double d) : I(i), J(j), K(k), dx(d) {}

    V3 bodyForce() const {   // _getConstantBodyForce (fluidsimulation.cpp:3363-3370)
        V3 bf;
        for (auto &f : bodyForces) bf = bf + f;
        return bf;
    }

    // ------------------------------------------------- initialize (2652)
    void initialize() {
        if (initialized) return;
        u.init(I + 1, J, K, 0.0f); v.init(I, J + 1, K, 0.0f); w.init(I, J, K + 1, 0.0f);
        vu.init(I + 1, J, K, 0); vv.init(I, J + 1, K, 0); vw.init(I, J, K + 1, 0);
        phi.init(I, J, K, 0.0f);
        float upper = (float)((double)((I + 1) + (J + 1) + (K + 1)) * dx);
        solidPhi.init(I + 1, J + 1, K + 1, upper);
        sdfRadius = 0.5 * 1.0 * dx * std::sqrt(3.0);      // _initializeParticleRadii (2644-2650)
        // _loadMarkerParticles (2773-2786): keep points inside the domain AABB
        double W = I * dx, H = J * dx, D = K * dx;
        for (auto &mp : loadQueue) {
            V3 p = divide(mp.p - V3(0, 0, 0), 1.0f);
            if (p.x >= 0.0f && p.y >= 0.0f && p.z >= 0.0f && p.x < 0.0 + W && p.y < 0.0 + H && p.z < 0.0 + D)
                parts.push_back(Particle{p, mp.v});
        }
        loadQueue.clear();
        initialized = true;
    }

    // Boundary AABB (fluidsimulation.cpp:2834-2839, aabb.cpp expand):
    // (0,0,0, I dx, J dx, K dx) shrunk by 3 dx + 1e-4 in total per axis.
    void boundaryAABB(double shrinkExtra, V3 &pos, double &wx, double &wy, double &wz) const {
        pos = V3(0, 0, 0);
        wx = I * dx; wy = J * dx; wz = K * dx;
        double v = -3 * dx - 1e-4;
        double h = 0.5 * v;
        pos = pos - V3((float)h, (float)h, (float)h);
        wx += v; wy += v; wz += v;
        if (shrinkExtra != 0.0) {
            double v2 = -shrinkExtra;
            double h2 = 0.5 * v2;
            pos = pos - V3((float)h2, (float)h2, (float)h2);
            wx += v2; wy += v2; wz += v2;
        }
    }

    // ------------------------------------------- solid level set (3028)
    // Domain walls: the boundary box mesh (_getTriangleMeshFromAABB,
    // fluidsimulation.cpp:2806-2832), exact band distances
    // (meshlevelset.cpp:1165-1230), signs from inside/outside, then negate
    // (fluidsimulation.cpp:2927-2935).
    void buildSolid() {
        V3 bp; double bw, bh, bd;
        boundaryAABB(0.0, bp, bw, bh, bd);
        V3 P = bp;
        V3 vert[8] = {
            V3(P.x, P.y, P.z), V3((float)(P.x + bw), P.y, P.z), V3((float)(P.x + bw), P.y, (float)(P.z + bd)),
            V3(P.x, P.y, (float)(P.z + bd)), V3(P.x, (float)(P.y + bh), P.z),
            V3((float)(P.x + bw), (float)(P.y + bh), P.z), V3((float)(P.x + bw), (float)(P.y + bh), (float)(P.z + bd)),
            V3(P.x, (float)(P.y + bh), (float)(P.z + bd))};
        int tris[12][3] = {{0, 1, 2}, {0, 2, 3}, {4, 7, 6}, {4, 6, 5}, {0, 3, 7}, {0, 7, 4},
                           {1, 5, 6}, {1, 6, 2}, {0, 4, 5}, {0, 5, 1}, {3, 2, 6}, {3, 6, 7}};
        int ni = I + 1, nj = J + 1, nk = K + 1;
        float upper = (float)((double)(ni + nj + nk) * dx);
        solidPhi.init(ni, nj, nk, upper);
        double invdx = 1.0 / dx;
        for (int t = 0; t < 12; t++) {
            V3 p = vert[tris[t][0]], q = vert[tris[t][1]], r = vert[tris[t][2]];
            double fi[3] = {p.x * invdx, q.x * invdx, r.x * invdx};
            double fj[3] = {p.y * invdx, q.y * invdx, r.y * invdx};
            double fk[3] = {p.z * invdx, q.z * invdx, r.z * invdx};
            auto lo = [&](double *f, int n) {
                return std::max(0, std::min(n - 1, int(std::fmin(f[0], std::fmin(f[1], f[2]))) - exactBand));
            };
            auto hi = [&](double *f, int n) {
                return std::max(0, std::min(n - 1, int(std::fmax(f[0], std::fmax(f[1], f[2]))) + exactBand + 1));
            };
            int i0 = lo(fi, ni), j0 = lo(fj, nj), k0 = lo(fk, nk);
            int i1 = hi(fi, ni), j1 = hi(fj, nj), k1 = hi(fk, nk);
            // distances are taken in the frame of the 10^3-node block holding
            // the node (meshlevelset.cpp:1114-1158)
            for (int k = k0; k <= k1; k++)
                for (int j = j0; j <= j1; j++)
                    for (int i = i0; i <= i1; i++) {
                        const int bw = 10;
                        V3 off = idxToPos(i / bw, j / bw, k / bw, (double)bw * dx);
                        V3 g = idxToPos(i % bw, j % bw, k % bw, dx);
                        float d = length(closestOnTriangle(g, p - off, q - off, r - off) - g);
                        if (d < solidPhi(i, j, k)) solidPhi(i, j, k) = d;
                    }
        }
        // inside the box mesh -> negative; then the domain level set is negated
        for (int k = 0; k < nk; k++)
            for (int j = 0; j < nj; j++)
                for (int i = 0; i < ni; i++) {
                    V3 g = idxToPos(i, j, k, dx);
                    bool inside = g.x > P.x && g.y > P.y && g.z > P.z && g.x < P.x + bw && g.y < P.y + bh &&
                                  g.z < P.z + bd;
                    float val = solidPhi(i, j, k);
                    if (inside) val = -val;
                    solidPhi(i, j, k) = -val;
                }
        // weight grid (fluidsimulation.cpp:3690-3730; meshlevelset.cpp:348-391)
        wU.init(I + 1, J, K, 0.0f); wV.init(I, J + 1, K, 0.0f); wW.init(I, J, K + 1, 0.0f);
        auto &S = solidPhi;
        for (int k = 0; k < K; k++)
            for (int j = 0; j < J; j++)
                for (int i = 0; i <= I; i++) {
                    float f = fraction4(S(i, j, k), S(i, j + 1, k), S(i, j, k + 1), S(i, j + 1, k + 1));
                    wU(i, j, k) = std::max(0.0f, std::min(1.0f - f, 1.0f));
                }
        for (int k = 0; k < K; k++)
            for (int j = 0; j <= J; j++)
                for (int i = 0; i < I; i++) {
                    float f = fraction4(S(i, j, k), S(i, j, k + 1), S(i + 1, j, k), S(i + 1, j, k + 1));
                    wV(i, j, k) = std::max(0.0f, std::min(1.0f - f, 1.0f));
                }
        for (int k = 0; k <= K; k++)
            for (int j = 0; j < J; j++)
                for (int i = 0; i < I; i++) {
                    float f = fraction4(S(i, j, k), S(i, j + 1, k), S(i + 1, j, k), S(i + 1, j + 1, k));
                    wW(i, j, k) = std::max(0.0f, std::min(1.0f - f, 1.0f));
                }
        solidBuilt = true;
    }

    // Near-solid coarse grid (fluidsimulation.cpp:3083-3126, gridutils.cpp:230-263)
    void buildNearSolid() {
        nearCell = nearFactor * dx;
        int gi = (int)std::ceil(I * dx / nearCell), gj = (int)std::ceil(J * dx / nearCell),
            gk = (int)std::ceil(K * dx / nearCell);
        nearSolid.init(gi, gj, gk, 0);
        float maxd = (float)(exactBand * dx);
        for (int k = 0; k < K; k++)
            for (int j = 0; j < J; j++)
                for (int i = 0; i < I; i++)
                    if (std::abs(solidPhi(i, j, k)) < maxd) nearSolid(i / nearFactor, j / nearFactor, k / nearFactor) = 1;
        int layers = (int)std::ceil((float)cfl / (float)nearFactor);
        for (int l = 0; l < layers; l++) {
            Grid<uint8_t> src = nearSolid;
            for (int k = 0; k < gk; k++)
                for (int j = 0; j < gj; j++)
                    for (int i = 0; i < gi; i++) {
                        if (!src(i, j, k)) continue;
                        int nb[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k}, {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
                        for (auto &n : nb)
                            if (nearSolid.in(n[0], n[1], n[2])) nearSolid(n[0], n[1], n[2]) = 1;
                    }
        }
    }

    // ------------------------------------------ liquid SDF (particlelevelset.cpp)
    // Blocks of 10^3 cells, particle lists per block, block-local float frame
    // (_computeSignedDistanceFromParticles :299-375, _computeGridCountDataThread
    // :477-532, _computeExactBandProducerThread :582-629).
    void computeLiquidSDF() {
        const int bw = 10;
        phi.fill((float)(3.0 * dx));
        if (parts.empty()) return;
        int bi = (I + bw - 1) / bw, bj = (J + bw - 1) / bw, bk = (K + bw - 1) / bw;
        float blockdx = (float)(bw * dx);
        Grid<uint8_t> active; active.init(bi, bj, bk, 0);
        for (auto &pt : parts) {
            GI g = posToIdx(pt.p, blockdx);
            if (active.in(g.i, g.j, g.k)) active(g.i, g.j, g.k) = 1;
        }
        feather26(active);
        float r = (float)sdfRadius;
        float sr = 2.0f * (float)sdfRadius;
        std::vector<std::vector<int>> lists =
            buildBlockLists(active, nthreads, [&](int n) { return parts[n].p; }, sr, blockdx);
        std::vector<int> work;   // blocks with particles, in block order
        for (int id = 0; id < (int)active.a.size(); id++)
            if (active.a[id] && !lists[id].empty()) work.push_back(id);
        parallel_ranges((int)work.size(), nthreads, [&](int w0, int w1) {
            for (int wq = w0; wq < w1; wq++) {
                    const int id = work[wq], i = id % bi, j = (id / bi) % bj, k = id / (bi * bj);
                    auto &L = lists[id];
                    float data[1000];
                    for (int q = 0; q < 1000; q++) data[q] = (float)(3.0 * dx);
                    V3 off = idxToPos(i, j, k, (double)bw * dx);
                    for (int n : L) {
                        V3 p = parts[n].p - off;
                        V3 pmin(p.x - sr, p.y - sr, p.z - sr), pmax(p.x + sr, p.y + sr, p.z + sr);
                        GI g0 = posToIdx(pmin, dx), g1 = posToIdx(pmax, dx);
                        g0.i = std::max(g0.i, 0); g0.j = std::max(g0.j, 0); g0.k = std::max(g0.k, 0);
                        g1.i = std::min(g1.i, bw - 1); g1.j = std::min(g1.j, bw - 1); g1.k = std::min(g1.k, bw - 1);
                        for (int c = g0.k; c <= g1.k; c++)
                            for (int b = g0.j; b <= g1.j; b++)
                                for (int a = g0.i; a <= g1.i; a++) {
                                    V3 gp = cellCenter(a, b, c, dx);
                                    float dist = length(gp - p) - r;
                                    int f = a + bw * (b + bw * c);
                                    if (dist < data[f]) data[f] = dist;
                                }
                    }
                    for (int q = 0; q < 1000; q++) {
                        int a = q % bw, b = (q / bw) % bw, c = q / (bw * bw);
                        int gi = i * bw + a, gj = j * bw + b, gk = k * bw + c;
                        if (phi.in(gi, gj, gk)) phi(gi, gj, gk) = data[q];
                    }
            }
        });
    }

    static void feather26(Grid<uint8_t> &g) {
        Grid<uint8_t> src = g;
        for (int k = 0; k < g.nk; k++)
            for (int j = 0; j < g.nj; j++)
                for (int i = 0; i < g.ni; i++) {
                    if (!src(i, j, k)) continue;
                    for (int c = -1; c <= 1; c++)
                        for (int b = -1; b <= 1; b++)
                            for (int a = -1; a <= 1; a++)
                                if (g.in(i + a, j + b, k + c)) g(i + a, j + b, k + c) = 1;
                }
    }

    // Which active blocks a point's search box overlaps, as the reference's
    // count pass decides it (simple case: box strictly inside its own block).
    // The block lists of all particles, each in ascending particle order (the
    // reference's count pass runs on threads over contiguous particle ranges
    // and concatenates them in range order, particlelevelset.cpp:435-580):
    // the threads fill lists of their own and the ranges are joined in order.
    template <class P>
    std::vector<std::vector<int>> buildBlockLists(const Grid<uint8_t> &active, int nt, P pos, float sr,
                                                  float blockdx) const {
        const int np = (int)parts.size();
        nt = std::max(1, std::min(nt, np));
        std::vector<std::vector<std::vector<int>>> part(nt, std::vector<std::vector<int>>(active.a.size()));
        std::vector<int> iv = splitRange(0, np, nt);
        parallel_ranges(nt, nt, [&](int t0, int t1) {
            for (int t = t0; t < t1; t++)
                for (int n = iv[t]; n < iv[t + 1]; n++) blockLists(pos(n), sr, blockdx, active, part[t], n);
        });
        std::vector<std::vector<int>> lists(active.a.size());
        parallel_ranges((int)lists.size(), nt, [&](int b0, int b1) {
            for (int b = b0; b < b1; b++) {
                size_t total = 0;
                for (int t = 0; t < nt; t++) total += part[t][b].size();
                lists[b].reserve(total);
                for (int t = 0; t < nt; t++) lists[b].insert(lists[b].end(), part[t][b].begin(), part[t][b].end());
            }
        });
        return lists;
    }

    static void blockLists(V3 p, float sr, float blockdx, const Grid<uint8_t> &active,
                           std::vector<std::vector<int>> &lists, int n) {
        GI bi = posToIdx(p, blockdx);
        V3 bp = idxToPos(bi.i, bi.j, bi.k, blockdx);
        auto blockId = [&](int i, int j, int k) -> long {
            if (!active.in(i, j, k) || !active(i, j, k)) return -1;
            return (long)active.idx(i, j, k);
        };
        if (p.x - sr > bp.x && p.y - sr > bp.y && p.z - sr > bp.z && p.x + sr < bp.x + blockdx &&
            p.y + sr < bp.y + blockdx && p.z + sr < bp.z + blockdx) {
            long id = blockId(bi.i, bi.j, bi.k);
            if (id >= 0) lists[id].push_back(n);
        } else {
            GI g0 = posToIdx((double)(p.x - sr), (double)(p.y - sr), (double)(p.z - sr), blockdx);
            GI g1 = posToIdx((double)(p.x + sr), (double)(p.y + sr), (double)(p.z + sr), blockdx);
            for (int c = g0.k; c <= g1.k; c++)
                for (int b = g0.j; b <= g1.j; b++)
                    for (int a = g0.i; a <= g1.i; a++) {
                        long id = blockId(a, b, c);
                        if (id >= 0) lists[id].push_back(n);
                    }
        }
    }

    // ParticleLevelSet::postProcessSignedDistanceField (particlelevelset.cpp:172-196)
    void postProcessSDF() {
        float eps = (float)(0.005 * dx);
        for (int k = 0; k < K; k++)
            for (int j = 0; j < J; j++)
                for (int i = 0; i < I; i++) {
                    if ((double)phi(i, j, k) < 0.5 * dx) {
                        const Grid<float> &S = solidPhi;
                        float cc = 0.125f * (S(i, j, k) + S(i + 1, j, k) + S(i, j + 1, k) + S(i + 1, j + 1, k) +
                                             S(i, j, k + 1) + S(i + 1, j, k + 1) + S(i, j + 1, k + 1) +
                                             S(i + 1, j + 1, k + 1));
                        if (cc < 0) phi(i, j, k) = (float)(-0.5f * dx);
                    }
                    float val = phi(i, j, k);
                    if (std::abs(val) < eps) phi(i, j, k) = val > 0 ? eps : -eps;
                }
    }

    // ------------------------------------------ P2G (velocityadvector.cpp:38-459)
    void p2g() {
        u.fill(0.0f); v.fill(0.0f); w.fill(0.0f);
        vu.fill(0); vv.fill(0); vw.fill(0);
        if (parts.empty()) return;
        p2gDir(0, u, vu);
        p2gDir(1, v, vv);
        p2gDir(2, w, vw);
    }

    void p2gDir(int dir, Grid<float> &G, Grid<uint8_t> &valid) {
        const int cw = 10;
        double chunkdx = dx * cw;
        V3 off = dir == 0 ? V3(0.0f, (float)(0.5 * dx), (float)(0.5 * dx))
               : dir == 1 ? V3((float)(0.5 * dx), 0.0f, (float)(0.5 * dx))
                          : V3((float)(0.5 * dx), (float)(0.5 * dx), 0.0f);
        int ni = G.ni, nj = G.nj, nk = G.nk;
        int bi = (ni + cw - 1) / cw, bj = (nj + cw - 1) / cw, bk = (nk + cw - 1) / cw;
        Grid<uint8_t> active; active.init(bi, bj, bk, 0);
        for (auto &pt : parts) {
            GI g = posToIdx(pt.p - off, chunkdx);
            if (active.in(g.i, g.j, g.k)) active(g.i, g.j, g.k) = 1;
        }
        feather26(active);
        float eps = 1e-6f;
        float sr = (float)(sdfRadius + eps);
        float blockdx = (float)chunkdx;
        std::vector<std::vector<int>> lists =
            buildBlockLists(active, nthreads, [&](int n) { return parts[n].p - off; }, sr, blockdx);
        float r = (float)sdfRadius;
        float rsq = r * r;
        float coef1 = (4.0f / 9.0f) * (1.0f / (r * r * r * r * r * r));
        float coef2 = (17.0f / 9.0f) * (1.0f / (r * r * r * r));
        float coef3 = (22.0f / 9.0f) * (1.0f / (r * r));
        std::vector<int> work;   // blocks with particles, in block order
        for (int id = 0; id < (int)active.a.size(); id++)
            if (active.a[id] && !lists[id].empty()) work.push_back(id);
        parallel_ranges((int)work.size(), nthreads, [&](int w0, int w1) {
            for (int wq = w0; wq < w1; wq++) {
                    const int id = work[wq], i = id % bi, j = (id / bi) % bj, k = id / (bi * bj);
                    auto &L = lists[id];
                    float sc[1000], wt[1000];
                    for (int q = 0; q < 1000; q++) sc[q] = wt[q] = 0.0f;
                    V3 boff = idxToPos(i, j, k, (double)cw * dx);
                    for (int n : L) {
                        V3 p = (parts[n].p - off) - boff;
                        float vel = dir == 0 ? parts[n].v.x : dir == 1 ? parts[n].v.y : parts[n].v.z;
                        V3 pmin(p.x - sr, p.y - sr, p.z - sr), pmax(p.x + sr, p.y + sr, p.z + sr);
                        GI g0 = posToIdx(pmin, dx), g1 = posToIdx(pmax, dx);
                        g0.i = std::max(g0.i, 0); g0.j = std::max(g0.j, 0); g0.k = std::max(g0.k, 0);
                        g1.i = std::min(g1.i, cw - 1); g1.j = std::min(g1.j, cw - 1); g1.k = std::min(g1.k, cw - 1);
                        for (int c = g0.k; c <= g1.k; c++)
                            for (int b = g0.j; b <= g1.j; b++)
                                for (int a = g0.i; a <= g1.i; a++) {
                                    V3 gp = idxToPos(a, b, c, dx);
                                    V3 dv = gp - p;
                                    float d2 = dot(dv, dv);
                                    if (d2 < rsq) {
                                        float wgt = 1.0f - coef1 * d2 * d2 * d2 + coef2 * d2 * d2 - coef3 * d2;
                                        int f = a + cw * (b + cw * c);
                                        sc[f] += wgt * vel;
                                        wt[f] += wgt;
                                    }
                                }
                    }
                    for (int q = 0; q < 1000; q++)
                        if (wt[q] > eps) sc[q] /= wt[q];
                    for (int q = 0; q < 1000; q++) {
                        int a = q % cw, b = (q / cw) % cw, c = q / (cw * cw);
                        int gi = i * cw + a, gj = j * cw + b, gk = k * cw + c;
                        if (G.in(gi, gj, gk)) {
                            G(gi, gj, gk) = sc[q];
                            if (wt[q] > eps) valid(gi, gj, gk) = 1;
                        }
                    }
            }
        });
    }

    // ------------------------------- extrapolation (gridutils.cpp:32-228)
    // Layered BFS: layer L fills unknown cells next to the cells known
    // before it with the mean of their finished neighbours; border cells of
    // the grid count as finished from the start.
    static void extrapolate(Grid<float> &G, const Grid<uint8_t> &valid, int layers, int nt) {
        const uint8_t UNKNOWN = 0, WAITING = 1, KNOWN = 2, DONE = 3;
        Grid<uint8_t> st; st.init(G.ni, G.nj, G.nk, UNKNOWN);
        for (int k = 0; k < G.nk; k++)
            for (int j = 0; j < G.nj; j++)
                for (int i = 0; i < G.ni; i++) {
                    if (onBorder(i, j, k, G.ni, G.nj, G.nk)) st(i, j, k) = DONE;
                    else if (valid(i, j, k)) st(i, j, k) = KNOWN;
                }
        std::vector<GI> cells;
        for (int l = 0; l < layers; l++) {
            cells.clear();
            for (int k = 0; k < G.nk; k++)
                for (int j = 0; j < G.nj; j++)
                    for (int i = 0; i < G.ni; i++) {
                        if (st(i, j, k) != KNOWN) continue;
                        GI nb[6] = {{i + 1, j, k}, {i - 1, j, k}, {i, j + 1, k}, {i, j - 1, k}, {i, j, k + 1}, {i, j, k - 1}};
                        for (auto &n : nb)
                            if (st(n.i, n.j, n.k) == UNKNOWN) { st(n.i, n.j, n.k) = WAITING; cells.push_back(n); }
                        st(i, j, k) = DONE;
                    }
            // the layer's cells read only DONE cells, which the layer does not write
            parallel_ranges((int)cells.size(), nt, [&](int c0, int c1) {
                for (int q = c0; q < c1; q++) {
                    const GI g = cells[q];
                    float sum = 0.0f;
                    int count = 0;
                    GI nb[6] = {{g.i + 1, g.j, g.k}, {g.i - 1, g.j, g.k}, {g.i, g.j + 1, g.k},
                                {g.i, g.j - 1, g.k}, {g.i, g.j, g.k + 1}, {g.i, g.j, g.k - 1}};
                    for (auto &n : nb)
                        if (st(n.i, n.j, n.k) == DONE) { sum += G(n.i, n.j, n.k); count++; }
                    G(g.i, g.j, g.k) = sum / (float)count;
                }
            });
            if (l != layers - 1)
                for (auto &g : cells) st(g.i, g.j, g.k) = KNOWN;
        }
    }

    void extrapolateMAC() {
        int layers = (int)std::ceil(cfl) + 2;    // fluidsimulation.cpp:3775-3779
        extrapolate(u, vu, layers, nthreads);
        extrapolate(v, vv, layers, nthreads);
        extrapolate(w, vw, layers, nthreads);
    }

    // ----------------------------- body forces (fluidsimulation.cpp:3450-3489)
    void applyBodyForce(double dt) {
        V3 bf = bodyForce();
        float eps = 1e-6f;
        if (std::fabs(bf.x) > eps) for (auto &x : u.a) x += (float)(bf.x * dt);
        if (std::fabs(bf.y) > eps) for (auto &x : v.a) x += (float)(bf.y * dt);
        if (std::fabs(bf.z) > eps) for (auto &x : w.a) x += (float)(bf.z * dt);
    }

    // ---------------------------------------------- pressure (pressuresolver.cpp)
    std::vector<double> lastPressureGrid, lastRhsGrid;

    double dotp(const std::vector<double> &x, const std::vector<double> &y) const {
        // BLAS::dot (pcgsolver/blaswrapper.h:36-64)
        int n = (int)x.size();
        int nt = (int)std::fmin(nthreads, std::ceil((float)n / 500000.0f));
        if (nt <= 1) {
            double s = 0;
            for (int i = 0; i < n; i++) s += x[i] * y[i];
            return s;
        }
        std::vector<int> iv = splitRange(0, n, nt);
        std::vector<double> parts_(nt, 0.0);
        parallel_ranges(nt, nt, [&](int t0, int t1) {   // one partition per thread
            for (int t = t0; t < t1; t++) {
                double part = 0;
                for (int i = iv[t]; i < iv[t + 1]; i++) part += x[i] * y[i];
                parts_[t] = part;
            }
        });
        double s = 0;
        for (int t = 0; t < nt; t++) s += parts_[t];
        return s;
    }
    static double absmax(const std::vector<double> &x) {
        double m = 0;
        for (double a : x) m = std::max(m, std::fabs(a));
        return m;
    }

    bool pressureSolve(double dt, std::vector<double> *pgridOut, std::vector<double> *rhsOut) {
        // fluid cells: interior cells with phi < 0 (pressuresolver.cpp:101-110)
        Grid<int> key; key.init(I, J, K, -1);
        std::vector<GI> cells;
        for (int k = 1; k < K - 1; k++)
            for (int j = 1; j < J - 1; j++)
                for (int i = 1; i < I - 1; i++)
                    if (phi(i, j, k) < 0) { key(i, j, k) = (int)cells.size(); cells.push_back(GI{i, j, k}); }
        int n = (int)cells.size();
        if (pgridOut) pgridOut->assign((size_t)I * J * K, 0.0);
        if (rhsOut) rhsOut->assign((size_t)I * J * K, 0.0);
        lastIters = 0; lastError = 0;
        // RHS (:580-669); solid face velocities are zero for the domain walls
        std::vector<double> b(n, 0.0);
        double factor = 1.0 / dx;
        for (int c = 0; c < n; c++) {
            int i = cells[c].i, j = cells[c].j, k = cells[c].k;
            double vR = wU(i + 1, j, k), vL = wU(i, j, k), vT = wV(i, j + 1, k), vB = wV(i, j, k);
            double vF = wW(i, j, k + 1), vK = wW(i, j, k);
            double div = 0.0;
            div += -factor * vR * u(i + 1, j, k);
            div += factor * vL * u(i, j, k);
            div += -factor * vT * v(i, j + 1, k);
            div += factor * vB * v(i, j, k);
            div += -factor * vF * w(i, j, k + 1);
            div += factor * vK * w(i, j, k);
            b[c] = div;
        }
        if (rhsOut) for (int c = 0; c < n; c++) (*rhsOut)[phi.idx(cells[c].i, cells[c].j, cells[c].k)] = b[c];
        double maxAbs = 0.0;
        for (double x : b) if (std::fabs(x) > maxAbs) maxAbs = std::fabs(x);
        if (maxAbs < tol) return true;

        // matrix (:723-808): 7-point rows, columns ascending
        std::vector<Row7> A(n);
        double mf = dt / (dx * dx);
        const double maxtheta = 25.0, eps = 1e-9;
        for (int c = 0; c < n; c++) {
            int i = cells[c].i, j = cells[c].j, k = cells[c].k;
            double vR = wU(i + 1, j, k), vL = wU(i, j, k), vT = wV(i, j + 1, k), vB = wV(i, j, k);
            double vF = wW(i, j, k + 1), vK = wW(i, j, k);
            double pc = phi(i, j, k);
            double diag = (vR + vL + vT + vB + vF + vK) * mf;
            struct Nb { int i, j, k; double vol; };
            Nb nb[6] = {{i + 1, j, k, vR}, {i - 1, j, k, vL}, {i, j + 1, k, vT}, {i, j - 1, k, vB}, {i, j, k + 1, vF}, {i, j, k - 1, vK}};
            int offcol[6]; double offval[6]; int noff = 0;
            for (auto &q : nb) {
                double pn = phi(q.i, q.j, q.k);
                if (pn < 0.0) {
                    int col = key(q.i, q.j, q.k);
                    if (col >= 0) { offcol[noff] = col; offval[noff] = -q.vol * mf; noff++; }
                } else {
                    double theta = pn / (pc + eps);
                    theta = std::max(-maxtheta, std::min(theta, maxtheta));
                    diag -= q.vol * mf * theta;
                }
            }
            diag = std::max(diag, 0.0);
            // insert sorted
            Row7 &R = A[c];
            R.nnz = 0;
            int order[7]; double vals[7]; int m = 0;
            for (int q = 0; q < noff; q++) { order[m] = offcol[q]; vals[m] = offval[q]; m++; }
            order[m] = c; vals[m] = diag; m++;
            for (int a = 0; a < m; a++)
                for (int bb = a + 1; bb < m; bb++)
                    if (order[bb] < order[a]) { std::swap(order[a], order[bb]); std::swap(vals[a], vals[bb]); }
            for (int a = 0; a < m; a++) { R.col[a] = order[a]; R.val[a] = vals[a]; }
            R.nnz = m;
        }

        LowerFactor<double> F;
        mic0_factor(A, F);
        auto precond = [&](const std::vector<double> &rhs, std::vector<double> &res) { mic0_apply(F, rhs, res); };
        auto spmv = [&](const std::vector<double> &x, std::vector<double> &out) {
            parallel_ranges(n, nthreads, [&](int i0, int i1) {
                for (int i = i0; i < i1; i++) {
                    out[i] = 0;
                    for (int q = 0; q < A[i].nnz; q++) out[i] += A[i].val[q] * x[A[i].col[q]];
                }
            });
        };
        auto addScaled = [&](float alpha, const std::vector<double> &x, std::vector<double> &y) {
            parallel_ranges(n, nthreads, [&](int i0, int i1) {
                for (int i = i0; i < i1; i++) y[i] += alpha * x[i];
            });
        };
        // PCGSolver::solve (pcgsolver.h:248-302)
        std::vector<double> x(n, 0.0), r = b, z(n), s(n);
        double resid = absmax(r);
        bool ok = false;
        int iterations = 0;
        if (resid == 0) { ok = true; }
        else {
            double ptol = std::max(tol, 1e-30) * resid;
            precond(r, z);
            double rho = dotp(z, r);
            if (rho == 0 || rho != rho) { ok = false; iterations = 0; }
            else {
                s = z;
                int it;
                for (it = 0; it < maxIter; it++) {
                    spmv(s, z);
                    double alpha = rho / dotp(s, z);
                    addScaled((float)alpha, s, x);
                    addScaled((float)-alpha, z, r);
                    resid = absmax(r);
                    if (resid <= ptol) { iterations = it + 1; ok = true; break; }
                    precond(r, z);
                    double rhoNew = dotp(z, r);
                    double beta = rhoNew / rho;
                    addScaled((float)beta, s, z);
                    s.swap(z);
                    rho = rhoNew;
                }
                if (!ok) iterations = it;
            }
        }
        lastIters = iterations;
        lastError = resid;
        bool accept = ok || (iterations == maxIter && resid < accTol);   // pressuresolver.cpp:810-840
        if (pgridOut) for (int c = 0; c < n; c++) (*pgridOut)[phi.idx(cells[c].i, cells[c].j, cells[c].k)] = x[c];
        if (!accept) return false;
        applyPressure(dt, cells, x);
        return true;
    }

    // _applySolutionToVelocityField / _applyPressureToVelocityFieldThread
    // (pressuresolver.cpp:842-1046), without surface tension
    void applyPressure(double dt, const std::vector<GI> &cells, const std::vector<double> &x) {
        Grid<float> P; P.init(I, J, K, 0.0f);
        for (size_t c = 0; c < cells.size(); c++) P(cells[c].i, cells[c].j, cells[c].k) = (float)x[c];
        Grid<uint8_t> fluid; fluid.init(I, J, K, 0);
        for (size_t q = 0; q < phi.a.size(); q++) fluid.a[q] = phi.a[q] < 0.0 ? 1 : 0;
        vu.fill(0); vv.fill(0); vw.fill(0);
        float factor = (float)(dt / dx);
        const float eps = 1e-6f;
        const double maxtheta = 25.0;
        auto clampf = [&](float t) { return (float)std::max(-maxtheta, std::min((double)t, maxtheta)); };
        auto face = [&](float &vel, uint8_t &valid, float wt, bool border, int ai, int aj, int ak, int bi, int bj, int bk) {
            if (wt > 0 && border) {
                float p1 = 0.0f, p2 = 0.0f;
                bool f1 = fluid(ai, aj, ak), f2 = fluid(bi, bj, bk);
                if (f1 && f2) { p1 = P(ai, aj, ak); p2 = P(bi, bj, bk); }
                else {
                    float phi1 = phi(ai, aj, ak), phi2 = phi(bi, bj, bk);
                    double tension = 0.0;
                    if (f1) {
                        float tp = clampf(phi2 / (phi1 + eps));
                        float tt = clampf((phi1 - phi2) / (phi1 + eps));
                        p1 = P(ai, aj, ak);
                        p2 = (float)(tt * tension + tp * p1);
                    } else {
                        float tp = clampf(phi1 / (phi2 + eps));
                        float tt = clampf((phi2 - phi1) / (phi2 + eps));
                        p2 = P(bi, bj, bk);
                        p1 = (float)(tt * tension + tp * p2);
                    }
                }
                vel += (float)(-factor * (p2 - p1));
                valid = 1;
            } else {
                vel = 0.0f;
            }
        };
        for (int k = 0; k < K; k++)
            for (int j = 0; j < J; j++)
                for (int i = 0; i <= I; i++) {
                    if (i == 0 || i == I - 1) continue;
                    bool border = (i == I) ? fluid(i - 1, j, k) : (fluid(i, j, k) || fluid(i - 1, j, k));
                    if (wU(i, j, k) > 0 && border)
                        face(u(i, j, k), vu(i, j, k), wU(i, j, k), border, i - 1, j, k, i, j, k);
                    else u(i, j, k) = 0.0f;
                }
        for (int k = 0; k < K; k++)
            for (int j = 0; j <= J; j++)
                for (int i = 0; i < I; i++) {
                    if (j == 0 || j == J - 1) continue;
                    bool border = (j == J) ? fluid(i, j - 1, k) : (fluid(i, j, k) || fluid(i, j - 1, k));
                    if (wV(i, j, k) > 0 && border)
                        face(v(i, j, k), vv(i, j, k), wV(i, j, k), border, i, j - 1, k, i, j, k);
                    else v(i, j, k) = 0.0f;
                }
        for (int k = 0; k <= K; k++)
            for (int j = 0; j < J; j++)
                for (int i = 0; i < I; i++) {
                    if (k == 0 || k == K - 1) continue;
                    bool border = (k == K) ? fluid(i, j, k - 1) : (fluid(i, j, k) || fluid(i, j, k - 1));
                    if (wW(i, j, k) > 0 && border)
                        face(w(i, j, k), vw(i, j, k), wW(i, j, k), border, i, j, k - 1, i, j, k);
                    else w(i, j, k) = 0.0f;
                }
    }

    // constrain (fluidsimulation.cpp:3884-3950): faces with zero weight take the
    // solid velocity (zero for the domain); partial faces blend with friction 0
    static void constrain(Grid<float> &G, const Grid<float> &W) {
        for (size_t q = 0; q < G.a.size(); q++) {
            if (W.a[q] == 0) G.a[q] = 0.0f;
            else if (W.a[q] < 1.0f) {
                float f = 0.0f;
                G.a[q] = f * 0.0f + (1.0f - f) * G.a[q];
            }
        }
    }

    // ------------------------------------ interpolation (macvelocityfield.cpp)
    static bool inGrid(double x, double y, double z, double dx, int i, int j, int k) {
        return x >= 0 && y >= 0 && z >= 0 && x < dx * i && y < dx * j && z < dx * k;
    }
    static double tri(const double p[8], double x, double y, double z) {
        return p[0] * (1 - x) * (1 - y) * (1 - z) + p[1] * x * (1 - y) * (1 - z) + p[2] * (1 - x) * y * (1 - z) +
               p[3] * (1 - x) * (1 - y) * z + p[4] * x * (1 - y) * z + p[5] * (1 - x) * y * z +
               p[6] * x * y * (1 - z) + p[7] * x * y * z;
    }
    // _interpolateLinearU/V/W (macvelocityfield.cpp:519-613)
    double interpFace(const Grid<float> &G, int dir, double x, double y, double z) const {
        if (!inGrid(x, y, z, dx, I, J, K)) return 0.0;
        if (dir != 0) x -= 0.5 * dx;
        if (dir != 1) y -= 0.5 * dx;
        if (dir != 2) z -= 0.5 * dx;
        double inv = 1.0 / dx;
        int i = (int)std::floor(x * inv), j = (int)std::floor(y * inv), k = (int)std::floor(z * inv);
        double gx = (double)i * dx, gy = (double)j * dx, gz = (double)k * dx;
        double ix = (x - gx) * (1 / dx), iy = (y - gy) * (1 / dx), iz = (z - gz) * (1 / dx);
        double p[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 0}, {1, 1, 1}};
        for (int q = 0; q < 8; q++)
            if (G.in(i + off[q][0], j + off[q][1], k + off[q][2])) p[q] = G(i + off[q][0], j + off[q][1], k + off[q][2]);
        return tri(p, ix, iy, iz);
    }
    V3 evalVel(const Grid<float> &gu, const Grid<float> &gv, const Grid<float> &gw, V3 p) const {
        double x = p.x, y = p.y, z = p.z;
        if (!inGrid(x, y, z, dx, I, J, K)) return V3();
        return V3((float)interpFace(gu, 0, x, y, z), (float)interpFace(gv, 1, x, y, z), (float)interpFace(gw, 2, x, y, z));
    }
    // Interpolation::trilinearInterpolate(vec3, dx, grid) (interpolation.cpp:72-113)
    float solidAt(V3 p) const {
        GI g = posToIdx(p, dx);
        V3 gp = idxToPos(g.i, g.j, g.k, dx);
        double inv = 1.0 / dx;
        double ix = (p.x - gp.x) * inv, iy = (p.y - gp.y) * inv, iz = (p.z - gp.z) * inv;
        double q[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 0}, {1, 1, 1}};
        for (int t = 0; t < 8; t++)
            if (solidPhi.in(g.i + off[t][0], g.j + off[t][1], g.k + off[t][2]))
                q[t] = solidPhi(g.i + off[t][0], g.j + off[t][1], g.k + off[t][2]);
        return (float)tri(q, ix, iy, iz);
    }
    // trilinearInterpolateGradient (interpolation.cpp:197-258)
    V3 solidGrad(V3 p) const {
        GI g = posToIdx(p, dx);
        V3 gp = idxToPos(g.i, g.j, g.k, dx);
        double inv = 1.0 / dx;
        double ix = (p.x - gp.x) * inv, iy = (p.y - gp.y) * inv, iz = (p.z - gp.z) * inv;
        auto at = [&](int a, int b, int c) -> float {
            return solidPhi.in(g.i + a, g.j + b, g.k + c) ? solidPhi(g.i + a, g.j + b, g.k + c) : 0.0f;
        };
        float v000 = at(0, 0, 0), v100 = at(1, 0, 0), v010 = at(0, 1, 0), v001 = at(0, 0, 1);
        float v101 = at(1, 0, 1), v011 = at(0, 1, 1), v110 = at(1, 1, 0), v111 = at(1, 1, 1);
        auto bil = [](double a, double b, double c, double d, double x, double y) {
            double l1 = (1 - x) * a + x * b;
            double l2 = (1 - x) * c + x * d;
            return (1 - y) * l1 + y * l2;
        };
        float ddx00 = v100 - v000, ddx10 = v110 - v010, ddx01 = v101 - v001, ddx11 = v111 - v011;
        float gxv = (float)bil(ddx00, ddx10, ddx01, ddx11, iy, iz);
        float ddy00 = v010 - v000, ddy10 = v110 - v100, ddy01 = v011 - v001, ddy11 = v111 - v101;
        float gyv = (float)bil(ddy00, ddy10, ddy01, ddy11, ix, iz);
        float ddz00 = v001 - v000, ddz10 = v101 - v100, ddz01 = v011 - v010, ddz11 = v111 - v110;
        float gzv = (float)bil(ddz00, ddz10, ddz01, ddz11, ix, iy);
        return V3(gxv, gyv, gzv);
    }

    // ------------------------------------------- G2P (fluidsimulation.cpp:4082-4092)
    void updateParticleVelocities() {
        parallel_ranges((int)parts.size(), nthreads, [&](int p0, int p1) {
            for (int q = p0; q < p1; q++) {
                Particle &pt = parts[q];
                V3 vPIC = evalVel(u, v, w, pt.p);
                V3 vFLIP = (pt.v + vPIC) - evalVel(su, sv, sw, pt.p);
                pt.v = (float)picRatio * vPIC + (float)(1 - picRatio) * vFLIP;
            }
        });
    }

    // ------------------------------------------- advection (4191-4296)
    V3 rk3(V3 p0, double dt) const {
        V3 k1 = evalVel(u, v, w, p0);
        V3 k2 = evalVel(u, v, w, p0 + (float)(0.5 * dt) * k1);
        V3 k3 = evalVel(u, v, w, p0 + (float)(0.75 * dt) * k2);
        return p0 + (float)(dt / 9.0f) * ((2.0f * k1 + 3.0f * k2) + 4.0f * k3);
    }

    struct Box { V3 pos; double w, h, d; };
    static bool boxInside(const Box &b, V3 p) {
        return p.x >= b.pos.x && p.y >= b.pos.y && p.z >= b.pos.z && p.x < b.pos.x + b.w && p.y < b.pos.y + b.h &&
               p.z < b.pos.z + b.d;
    }
    static V3 boxNearest(const Box &b, V3 p) {
        if (boxInside(b, p)) return p;
        V3 mn = b.pos;
        V3 mx = b.pos + V3((float)b.w, (float)b.h, (float)b.d);
        double eps = 1e-6;
        p.x = std::fmax(p.x, mn.x); p.y = std::fmax(p.y, mn.y); p.z = std::fmax(p.z, mn.z);
        p.x = (float)std::fmin((double)p.x, mx.x - eps);
        p.y = (float)std::fmin((double)p.y, mx.y - eps);
        p.z = (float)std::fmin((double)p.z, mx.z - eps);
        return p;
    }
    bool nearAt(GI g) const { return nearSolid.in(g.i, g.j, g.k) && nearSolid(g.i, g.j, g.k); }

    V3 resolveCollision(V3 oldp, V3 newp, const Box &boundary) const {
        GI gg = posToIdx(newp, dx);
        if (!inRange(gg.i, gg.j, gg.k, I, J, K)) newp = boxNearest(boundary, newp);
        GI og = posToIdx(oldp, nearCell), ng = posToIdx(newp, nearCell);
        if (!nearAt(og) && !nearAt(ng)) return newp;
        float eps = 1e-6f;
        float stepDist = stepFactor * (float)dx;
        float travel = length(newp - oldp);
        if (travel < eps) return newp;
        int nsteps = (int)std::ceil(travel / stepDist);
        V3 dir = normalize(newp - oldp);
        V3 last = oldp, cur;
        bool found = false;
        float cphi = 0.0f;
        for (int s = 0; s < nsteps; s++) {
            if (s == nsteps - 1) cur = newp;
            else cur = oldp + ((float)(s + 1) * stepDist) * dir;
            float ph = solidAt(cur);
            if (ph < 0.0f || !boxInside(boundary, cur)) { cphi = ph; found = true; break; }
            last = cur;
        }
        if (!found) return newp;
        V3 res;
        float maxDist = (float)(cfl * dx);
        V3 g = solidGrad(cur);
        if (length(g) > eps) {
            g = normalize(g);
            res = cur - (float)(cphi - solidBuffer * dx) * g;
            float rphi = solidAt(res);
            float rd = length(res - cur);
            if (rphi < 0 || rd > maxDist) res = last;
        } else {
            res = last;
        }
        if (!boxInside(boundary, res)) {
            V3 orig = res;
            res = boxNearest(boundary, res);
            float rphi = solidAt(res);
            float rd = length(res - orig);
            if (rphi < 0.0f || rd > maxDist) res = last;
        }
        return res;
    }

    Box collisionBox() const {
        Box b;
        boundaryAABB(0.0, b.pos, b.w, b.h, b.d);
        double v2 = -(solidBuffer * dx);
        double h2 = 0.5 * v2;
        b.pos = b.pos - V3((float)h2, (float)h2, (float)h2);
        b.w += v2; b.h += v2; b.d += v2;
        return b;
    }

    void advance(double dt, std::vector<V3> *posAdv) {
        Box boundary = collisionBox();
        std::vector<V3> out(parts.size());
        parallel_ranges((int)parts.size(), nthreads, [&](int p0, int p1) {
            for (int q = p0; q < p1; q++) out[q] = resolveCollision(parts[q].p, rk3(parts[q].p, dt), boundary);
        });
        for (size_t q = 0; q < parts.size(); q++) parts[q].p = out[q];
        if (posAdv) *posAdv = out;
        removeParticles(frameDt);
    }

    // _getMarkerParticleSpeedLimit / _removeMarkerParticles (4298-4353)
    float speedLimit(double dt) const {
        double step = cfl * dx / dt;
        std::vector<int> counts(maxFrameSteps, 0);
        for (auto &pt : parts) {
            double speed = (double)length(pt.v);
            int idx = (int)std::fmin(std::floor(speed / step), maxFrameSteps - 1);
            counts[idx]++;
        }
        int maxRemoval = (int)std::fmin((int)((double)parts.size() * maxRemovePct), maxRemoveAbs);
        double maxspeed = maxFrameSteps * step;
        int cur = 0;
        for (int i = (int)counts.size() - 1; i > 0; i--) {
            if (cur + counts[i] > maxRemoval) break;
            cur += counts[i];
            maxspeed = i * step;
        }
        return (float)maxspeed;
    }
    void removeParticles(double dt) {
        Grid<int> count; count.init(I, J, K, 0);
        float maxspeed = speedLimit(dt);
        double maxsq = maxspeed * maxspeed;
        std::vector<Particle> keep;
        keep.reserve(parts.size());
        for (auto &pt : parts) {
            if (solidAt(pt.p) < 0.0f) continue;
            GI g = posToIdx(pt.p, dx);
            if (count(g.i, g.j, g.k) >= maxPerCell) continue;
            count(g.i, g.j, g.k) += 1;
            if (dot(pt.v, pt.v) > maxsq) continue;
            keep.push_back(pt);
        }
        parts.swap(keep);
    }

    // -------------------------------------------------- time stepping (5529-5845)
    double maxParticleSpeed() const {
        double m = 0.0;
        for (auto &pt : parts) {
            double d = dot(pt.v, pt.v);
            if (d > m) m = d;
        }
        return std::sqrt(m);
    }
    double nextTimeStep(double dt) const {
        double maxu;
        if (frame == 0 && stepNumber == 0) {
            V3 bf = bodyForce();
            maxu = 0.0 + length(bf) * dt;
        } else {
            maxu = maxParticleSpeed();
        }
        maxu = std::fmax(0.0, maxu);
        return cfl * dx / (maxu + 1e-6);
    }

    void stepFluid(double dt, OrcStageDump *d) {
        auto dumpMac = [&](float *a, float *b, float *c, const Grid<float> &x, const Grid<float> &y, const Grid<float> &z) {
            if (!a) return;
            std::memcpy(a, x.a.data(), x.a.size() * 4);
            std::memcpy(b, y.a.data(), y.a.size() * 4);
            std::memcpy(c, z.a.data(), z.a.size() * 4);
        };
        if (d && d->n_before) *d->n_before = (int)parts.size();
        // obstacles: static walls are built once; nothing happens without particles
        if (!solidBuilt && !parts.empty()) { buildSolid(); buildNearSolid(); }
        if (!solidBuilt) { solidPhi.fill((float)((double)((I + 1) + (J + 1) + (K + 1)) * dx)); }
        if (nearSolid.a.empty()) buildNearSolid();
        computeLiquidSDF();
        if (solidBuilt) postProcessSDF();
        else { // no solid: post-process against the upper-bound field (no cell is solid)
            float eps = (float)(0.005 * dx);
            for (auto &x : phi.a) if (std::abs(x) < eps) x = x > 0 ? eps : -eps;
        }
        if (d && d->phi) std::memcpy(d->phi, phi.a.data(), phi.a.size() * 4);
        p2g();
        if (d && d->vu_p2g) {
            std::memcpy(d->vu_p2g, vu.a.data(), vu.a.size());
            std::memcpy(d->vv_p2g, vv.a.data(), vv.a.size());
            std::memcpy(d->vw_p2g, vw.a.data(), vw.a.size());
        }
        if (!parts.empty()) extrapolateMAC();
        if (d) dumpMac(d->u_p2g, d->v_p2g, d->w_p2g, u, v, w);
        su = u; sv = v; sw = w;
        applyBodyForce(dt);
        if (d) dumpMac(d->u_force, d->v_force, d->w_force, u, v, w);
        if (!solidBuilt) buildSolid();
        std::vector<double> pg, rh;
        bool want = d && (d->pressure || d->rhs);
        pressureSolve(dt, want ? &pg : nullptr, want ? &rh : nullptr);
        if (d && d->pressure) for (size_t q = 0; q < pg.size(); q++) d->pressure[q] = (float)pg[q];
        if (d && d->rhs) for (size_t q = 0; q < rh.size(); q++) d->rhs[q] = rh[q];
        if (d && d->pcg_iters) *d->pcg_iters = lastIters;
        if (d && d->pcg_error) *d->pcg_error = lastError;
        extrapolateMAC();
        if (d) dumpMac(d->u_press, d->v_press, d->w_press, u, v, w);
        constrain(su, wU); constrain(sv, wV); constrain(sw, wW);
        constrain(u, wU); constrain(v, wV); constrain(w, wW);
        if (d) dumpMac(d->u_final, d->v_final, d->w_final, u, v, w);
        if (d) dumpMac(d->u_saved, d->v_saved, d->w_saved, su, sv, sw);
        updateParticleVelocities();
        if (d && d->vel_g2p)
            for (size_t q = 0; q < parts.size(); q++) {
                d->vel_g2p[3 * q] = parts[q].v.x; d->vel_g2p[3 * q + 1] = parts[q].v.y; d->vel_g2p[3 * q + 2] = parts[q].v.z;
            }
        std::vector<V3> pa;
        advance(dt, (d && d->pos_adv) ? &pa : nullptr);
        if (d && d->pos_adv)
            for (size_t q = 0; q < pa.size(); q++) {
                d->pos_adv[3 * q] = pa[q].x; d->pos_adv[3 * q + 1] = pa[q].y; d->pos_adv[3 * q + 2] = pa[q].z;
            }
    }

    void update(double dt, OrcStageDump *d) {
        double epsdt = 1e-6;
        bool zeroLength = dt < epsdt;
        dt = std::max(dt, epsdt);
        frameDt = dt;
        frameRemaining = dt;
        stepNumber = 0;
        bool skipped = zeroLength && outputInitialized;
        double substep = frameDt / (double)minFrameSteps;
        double eps = 1e-9;
        do {
            stepDt = std::fmin(nextTimeStep(dt), frameRemaining);
            double done = frameDt - frameRemaining;
            double limit = (stepNumber + 1) * substep;
            if (done + stepDt > limit) stepDt = std::fmin(substep, frameRemaining);
            if (stepNumber == maxFrameSteps - 1) stepDt = frameRemaining;
            frameRemaining -= stepDt;
            if (!skipped) stepFluid(stepDt, d);
            d = nullptr;  // stage dumps cover the first substep only
            stepNumber++;
        } while (frameRemaining > eps);
        lastSubsteps = stepNumber;
        outputInitialized = true;
        frame++;
    }
};

}  // namespace orc

using orc::Sim;

extern "C" {

void *orc_create(int i, int j, int k, double dx) { return new Sim(i, j, k, dx); }
void orc_destroy(void *h) { delete (Sim *)h; }
void orc_set_threads(void *h, int n) { ((Sim *)h)->nthreads = n < 1 ? 1 : n; }
void orc_set_pic_ratio(void *h, double r) { ((Sim *)h)->picRatio = r; }
void orc_add_body_force(void *h, double x, double y, double z) {
    ((Sim *)h)->bodyForces.push_back(orc::V3((float)x, (float)y, (float)z));
}
void orc_set_cfl(void *h, int c) { ((Sim *)h)->cfl = c; }
void orc_set_pressure_tol(void *h, double t) { ((Sim *)h)->tol = t; }
void orc_set_pressure_maxiter(void *h, int n) { ((Sim *)h)->maxIter = n; }
void orc_load_particles(void *h, int n, const float *pos, const float *vel) {
    Sim *s = (Sim *)h;
    for (int q = 0; q < n; q++)
        s->loadQueue.push_back(orc::Particle{orc::V3(pos[3 * q], pos[3 * q + 1], pos[3 * q + 2]),
                                             orc::V3(vel[3 * q], vel[3 * q + 1], vel[3 * q + 2])});
}
void orc_initialize(void *h) { ((Sim *)h)->initialize(); }
void orc_update(void *h, double dt) { ((Sim *)h)->update(dt, nullptr); }
int orc_update_staged(void *h, double dt, OrcStageDump *d) {
    Sim *s = (Sim *)h;
    if (!s->initialized) return -2;
    double step = std::fmin(s->nextTimeStep(std::max(dt, 1e-6)), std::max(dt, 1e-6));
    if (step < std::max(dt, 1e-6)) return -1;
    s->update(dt, d);
    return 0;
}
int orc_num_particles(void *h) { return (int)((Sim *)h)->parts.size(); }
void orc_get_particles(void *h, float *pos, float *vel) {
    Sim *s = (Sim *)h;
    for (size_t q = 0; q < s->parts.size(); q++) {
        if (pos) { pos[3 * q] = s->parts[q].p.x; pos[3 * q + 1] = s->parts[q].p.y; pos[3 * q + 2] = s->parts[q].p.z; }
        if (vel) { vel[3 * q] = s->parts[q].v.x; vel[3 * q + 1] = s->parts[q].v.y; vel[3 * q + 2] = s->parts[q].v.z; }
    }
}
void orc_get_liquid_phi(void *h, float *out) {
    Sim *s = (Sim *)h;
    std::memcpy(out, s->phi.a.data(), s->phi.a.size() * 4);
}
void orc_get_solid_phi(void *h, float *out) {
    Sim *s = (Sim *)h;
    if (!s->solidBuilt) s->buildSolid();
    std::memcpy(out, s->solidPhi.a.data(), s->solidPhi.a.size() * 4);
}
void orc_get_mac(void *h, float *u, float *v, float *w) {
    Sim *s = (Sim *)h;
    std::memcpy(u, s->u.a.data(), s->u.a.size() * 4);
    std::memcpy(v, s->v.a.data(), s->v.a.size() * 4);
    std::memcpy(w, s->w.a.data(), s->w.a.size() * 4);
}
void orc_get_weights(void *h, float *wu, float *wv, float *ww) {
    Sim *s = (Sim *)h;
    if (!s->solidBuilt) s->buildSolid();
    std::memcpy(wu, s->wU.a.data(), s->wU.a.size() * 4);
    std::memcpy(wv, s->wV.a.data(), s->wV.a.size() * 4);
    std::memcpy(ww, s->wW.a.data(), s->wW.a.size() * 4);
}
void orc_get_near_solid(void *h, int *dims, uint8_t *out) {
    Sim *s = (Sim *)h;
    if (!s->solidBuilt) s->buildSolid();
    if (s->nearSolid.a.empty()) s->buildNearSolid();
    dims[0] = s->nearSolid.ni; dims[1] = s->nearSolid.nj; dims[2] = s->nearSolid.nk;
    if (out) std::memcpy(out, s->nearSolid.a.data(), s->nearSolid.a.size());
}
int orc_last_pcg_iters(void *h) { return ((Sim *)h)->lastIters; }
double orc_last_pcg_error(void *h) { return ((Sim *)h)->lastError; }
int orc_frame_substeps(void *h) { return ((Sim *)h)->lastSubsteps; }

}  // extern "C"

using namespace orc;

extern "C" {
// The MIC(0) preconditioner on its own (unit checks of the factor and the
// sweeps against the reference's routines).  invdiag: n doubles per cell
// (0 off the system); lower: 3 doubles per cell, the scaled factor entries
// of the cell's column towards its +x, +y, +z rows (0 where absent).
int orc_mic0_factor(int I, int J, int K, const uint8_t *fluid, const double *rows7, double *invdiag, double *lower) {
    std::vector<Row7> A;
    std::vector<int> cellOf, rowOf;
    unit_system(I, J, K, fluid, rows7, A, cellOf, rowOf);
    LowerFactor<double> F;
    mic0_factor(A, F);
    const size_t nc = (size_t)I * J * K;
    std::fill(invdiag, invdiag + nc, 0.0);
    if (lower) std::fill(lower, lower + 3 * nc, 0.0);
    const long long step[3] = {1, (long long)I, (long long)I * J};
    for (size_t c = 0; c < cellOf.size(); c++) {
        const long long t = cellOf[c];
        invdiag[t] = F.invdiag[c];
        if (!lower) continue;
        for (int p = F.colstart[c]; p < F.colstart[c + 1]; p++) {
            const long long row = cellOf[F.rowidx[p]];
            for (int q = 0; q < 3; q++)
                if (row == t + step[q]) lower[3 * t + q] = F.lval[p];
        }
    }
    return (int)cellOf.size();
}

// z = M^-1 r in FP32 with the factor given per cell as {invdiag, L+x, L+y,
// L+z} (floats), the sweeps in the reference's order.
int orc_mic0_precondition_f32(int I, int J, int K, const uint8_t *fluid, const float *factor, const float *r,
                              float *z) {
    const size_t nc = (size_t)I * J * K;
    std::vector<int> rowOf(nc, -1), cellOf;
    for (size_t t = 0; t < nc; t++)
        if (fluid[t]) { rowOf[t] = (int)cellOf.size(); cellOf.push_back((int)t); }
    const int n = (int)cellOf.size();
    LowerFactor<float> F;
    F.invdiag.assign(n, 0.0f);
    F.colstart.assign(n + 1, 0);
    const long long step[3] = {1, (long long)I, (long long)I * J};
    for (int c = 0; c < n; c++) {
        const long long t = cellOf[c];
        F.colstart[c] = (int)F.rowidx.size();
        F.invdiag[c] = factor[4 * t];
        for (int q = 0; q < 3; q++) {
            const long long nb = t + step[q];
            if (nb < (long long)nc && fluid[nb]) { F.rowidx.push_back(rowOf[nb]); F.lval.push_back(factor[4 * t + 1 + q]); }
        }
    }
    F.colstart[n] = (int)F.rowidx.size();
    std::vector<float> rhs(n), res;
    for (int c = 0; c < n; c++) rhs[c] = r[cellOf[c]];
    mic0_apply(F, rhs, res);
    std::fill(z, z + nc, 0.0f);
    for (int c = 0; c < n; c++) z[cellOf[c]] = res[c];
    return n;
}
}  // extern "C"
