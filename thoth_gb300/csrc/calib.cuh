// calib.cuh — LSV leverage calibration (calib.cu): kernel arguments, launcher, and the
// host-side jump-ahead of the reference Rng (xoshiro256++), shared with thoth_gpu.cu.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "exact.cuh"

constexpr int CALIB_THREADS = 128;
constexpr int CALIB_MAX_BINS = 128;
constexpr int CALIB_JUMP_BITS = 40; // x^(2^i) mod chi for i < 40: particle offsets below 2^40

struct CalibArgs {
    int P, n, points, bins, min_count;
    double s0, ln_s0, v0, kappa, theta, xi, rho, min_cv, lmin, lmax;
    const double* dt;        // [n] year fraction of the step into date k (dt[0] unused)
    const double* carry;     // [n] cumulative carry of date k minus date k-1
    const double* qe_e;      // [n] exp(-kappa dt[k]), rounded on the host like the reference
    const double* ln_step;   // [n]
    const int64_t* offset;   // [n]
    const double* local_vol; // [n][points]
    double* lev;             // [n][points] out
    double *spot, *var, *lns; // [P] the ensemble
    uint64_t* rng;           // [4][P] each particle's Rng state
    const uint64_t* jpow;    // [CALIB_JUMP_BITS][4] x^(2^i) mod chi
    // the jump from a particle's draws of one date to the next (2P - 2 draws) as a nibble
    // table of its GF(2) matrix: jtab[(n 16 + v) 4 + w] = word w of the jump of the state
    // whose nibble n is v and other bits 0 (64 nibbles x 16 values x 32 bytes, 32 KB)
    const uint64_t* jtab;
    uint64_t seed_state[4];  // the Rng state after seeding
    // per-date totals the CTAs add into with integer atomics (order-independent, exact):
    long long *kmin, *kmax;  // [n] order-preserving integer keys of the extremes of ln S
                             // (initialised to 0x7f.. / 0x80.. bytes: neutral for min / max)
    Fx128* vsum;             // [n] sum of v (zero at launch)
    unsigned* bcnt;          // [n][bins] particles per bin (zero at launch)
    Fx128* bsum;             // [n][bins] sum of v per bin (zero at launch)
    double* bc;              // [4] published: min ln S, bin width, ensemble mean of v, degenerate
    unsigned *bar, *done;    // arrivals and releases, all rounds (zero at launch)
    int* status;             // 0 ok, 2 a wait timed out, 3 a sum out of range
};

constexpr size_t CALIB_JTAB_WORDS = 64 * 16 * 4;

int calib_max_grid(int sms, size_t smem);
cudaError_t launch_calib(const CalibArgs& A, int grid, size_t smem, cudaStream_t st);

// host: the reference Rng's transition, seeding, and jump polynomials
void xo_seed_state(uint64_t seed, uint64_t s[4]);
void xo_advance(uint64_t s[4]); // one transition of the state (no output)
// x^d mod chi, with chi the transition's characteristic polynomial (found once by
// Berlekamp-Massey); false if chi could not be found (never for xoshiro256)
bool xo_jump_poly(uint64_t d, uint64_t out[4]);
void xo_apply_jump(const uint64_t poly[4], uint64_t s[4]);
// the nibble table of the jump poly (CALIB_JTAB_WORDS words, layout of CalibArgs::jtab)
void xo_jump_table(const uint64_t poly[4], uint64_t* tab);

// The book kernel's Gaussians beyond the Sobol budget: the reference's PathGenerator::NextPath
// (path_generator.cpp:139-157) draws them from one Rng seeded with the pricing's seed, path
// after path, dt of them a path in dimension order. out[d][p] (d < dt, p < paths) is the
// d-th of path p, rounded to float. tail_normals_prepare uploads the jump polynomials to the
// current device once (call it before any stream capture).
cudaError_t tail_normals_prepare();
cudaError_t launch_tail_normals(uint64_t seed, int dt, int64_t paths, float* out, cudaStream_t st);
