// Particle readback in the reference's order (getMarkerParticlePositionData,
// src/engine/fluidsimulation.cpp:2408-2420): particles live sorted by cell;
// their ids are their ranks in the reference's (load) order, which removal
// only thins out.  Rank of each survivor = number of surviving ids below
// its own: flag ids, exclusive scan, scatter to packed xyz.
#include "flip_device.cuh"

namespace flip {

namespace {

__global__ void k_flag_ids(const unsigned int *ids, int n, int *flags) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) flags[ids[t]] = 1;
}

__global__ void k_scatter_xyz(ParticleSoA p, int n, const int *rank, float *pos, float *vel) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    long long o = 3LL * rank[p.id[t]];
    if (pos) { pos[o] = p.px[t]; pos[o + 1] = p.py[t]; pos[o + 2] = p.pz[t]; }
    if (vel) { vel[o] = p.vx[t]; vel[o + 1] = p.vy[t]; vel[o + 2] = p.vz[t]; }
}

__global__ void k_renumber_ids(unsigned int *ids, int n, const int *rank) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) ids[t] = (unsigned int)rank[ids[t]];
}

}  // namespace

// Ids renumbered to their ranks (0..n-1), which keeps every order the ids
// define; used when emission and removal have spread them out.
void launch_compact_ids(const ParticleSoA &p, int n, int idSpace, int *flags, int *rank, int *scratch, int *total,
                        cudaStream_t s) {
    cudaMemsetAsync(flags, 0, (size_t)(idSpace + 1) * sizeof(int), s);
    if (n > 0) { FLIP_COUNT(1); k_flag_ids<<<div_up(n, 256), 256, 0, s>>>(p.id, n, flags); }
    launch_scan_cells(flags, idSpace, rank, scratch, total, s);
    if (n > 0) { FLIP_COUNT(1); k_renumber_ids<<<div_up(n, 256), 256, 0, s>>>(p.id, n, rank); }
}

void launch_readback_order(const ParticleSoA &p, int n, int idSpace, int *flags, int *rank, int *scratch,
                           int *total, float *pos, float *vel, cudaStream_t s) {
    cudaMemsetAsync(flags, 0, (size_t)(idSpace + 1) * sizeof(int), s);
    if (n > 0) { FLIP_COUNT(1); k_flag_ids<<<div_up(n, 256), 256, 0, s>>>(p.id, n, flags); }
    launch_scan_cells(flags, idSpace, rank, scratch, total, s);
    if (n > 0) { FLIP_COUNT(1); k_scatter_xyz<<<div_up(n, 256), 256, 0, s>>>(p, n, rank, pos, vel); }
}

}  // namespace flip
