// yk_internal.h -- structures shared by the host runtime and the kernels.
// Device tables are plain structs in device memory; kernels get them through
// small by-value argument structs.
#pragma once

#include <stdint.h>

#include "yukawa.h"

#ifdef __CUDACC__
#define YK_HD __host__ __device__
#else
#define YK_HD
#endif

namespace yk {

constexpr int kBlock = 256;   // threads per block of the site kernels
constexpr int kTile = 256;    // lattice sites per tile (one per thread)
constexpr int kMaxFFT = 4096; // longest FFT edge handled in shared memory
constexpr int kMaxDFT = 256;  // longest non-power-of-two edge (direct DFT)
constexpr int kMaxTilesPerBlock = 4096;  // tiles one CG block may own
constexpr int kMaxGrid = 2048;           // blocks of a CG launch (neighbour flags allocated)
constexpr int kEobMaxSystems = 1024;     // systems of one batched even-odd solve
constexpr int kFlagStride = 32;          // one 128-byte line per neighbour flag

// Grid barrier of the CG kernel: arrivals are counted (monotonically within a
// solve) on one line; the last block to arrive finishes the reduction and
// publishes the grid word (active systems, reliable-update flag) stamped with
// the barrier's generation on another.
struct GridBarrier {
    unsigned arrive;
    unsigned pad0[31];
    unsigned long long gword;
    unsigned long long pad1[15];
    // mixed-precision single-system solves: fixed-point sums of the four
    // reduced values, three rotating buffers, each value on its own 128-byte line
    long long fsum[3][4][16];
};

// One linear system (chain, right-hand side) of a batched CG solve.
struct SysDev {
    int chain, rhs;
    int Nt, Nx, V;
    int tile0, ntiles;   // tiles of this system in the tile table
    double m0, g, r;     // Dirac parameters of the chain
    const double* sigma; // the chain's scalar field
    const double* pi;    // the chain's pions (3 x V doubles) on complex systems, or null
    // FP64 vectors (K real planes per spinor entry)
    double* b;           // right-hand side (eta)
    double* x;           // solution
    double* r64[2];      // residual, double-buffered (FP64 solver)
    double* p64[2];      // search directions, double-buffered
    double* t64;         // D p (or D x in reliable updates)
    double* Ap64;        // D^dag D p
    // FP32 vectors (mixed solver)
    float* r32[2];       // residual, double-buffered
    float* p32[2];       // search directions, double-buffered
    float* t32;          // D p
    float* Ap32;         // D^dag D p
    float* xs32;         // solution increment since the last reliable update
    float* diag32;       // 2r + m0 + g sigma per site (one float)
    double* dinv;        // even-odd views: 1 / (2r + m0 + g sigma) on the odd sites (compact)
    float* v32;          // batched even-odd views: v = S^dag p (even, compact)
    float* w32;          // and w, later u (odd, compact)
    // noise generation for b: kind/rhs of the Philox stream, or gen = 0
    int gen_eta;
    uint64_t seed;
    const int64_t* step; // device step counter of the chain
    // eta of the step's systems (kind 2) generated one step ahead, by step
    // parity, with the step each buffer holds (null: never generated ahead)
    double* eta_ahead[2];
    int64_t* eta_tag;
};

// Per-tile reduction slot of the CG kernel: |r|^2, |Ap|^2, <p, Ap> (re, im),
// <r, Ap> (re, im); after a reliable update |r|^2 and <r, p> of the FP64
// residual.  FP64 solver: FP64 sums; mixed solver: float-float (hi, lo) sums.
union __align__(16) Partial {
    double d[6];
    float2 f[6];
};

// Per-system CG scalars.  Written only by the block that completes a grid
// reduction (one at a time), read by the host after the solve.
struct CGState {
    double rr, rr0;      // last |r|^2, |b|^2
    double rr_prev;      // |r|^2 of the previous iteration (mixed: beta after a reliable update)
    double stop2;        // stopping threshold on |r|^2 (tol^2, or tol^2 |b|^2)
    double rmax2;        // largest |r|^2 since the last reliable update (mixed)
    int active;
    int iters;
    int converged;
    int status;
    int n_ru;            // reliable updates (mixed)
    int mode;            // the system's mode in the pass that follows
    int chi_ready;       // the solve ended in a reliable update: t64 holds D_first x of the final x
};

// Per-system coefficients of the next pass (alpha: x += alpha p, r -= alpha A p;
// beta, c: p = c r + beta p; the mode), published with each grid reduction as
// twelve 64-bit words, each carrying 32 bits of payload and the barrier
// generation in its high half.
struct __align__(16) CGCoef {
    unsigned long long w[12];
};

struct CGArgs {
    SysDev* sys;
    int sys_first, sys_count;   // systems taking part in this solve
    const int2* tiles;          // (system, first site) of the whole table
    int tile_begin, tile_end;   // tiles of this solve
    int eta_kind;               // Philox stream kind of generated right-hand sides
    CGState* st;
    Partial* partial;    // one per tile
    CGCoef* coef;        // one per system
    unsigned* flags;     // kMaxGrid neighbour flags, kFlagStride apart
    int tiles_per_block; // contiguous tile range of each block (set by the launcher)
    int grid;            // blocks of the launch (set by the launcher)
    GridBarrier* bar;
    int* err;
    int* n_active;
    int* any_ru;
    int max_iter;
    int mtype;           // YK_DAGGER: A = D^dag D;  YK_NORMAL: A = D D^dag
    int tol_mode;
    double tol;
    int reliable_every;
    double reliable_delta;
    int solo_nt, solo_nx;   // lattice of a single-system solve (0: not given; the halo kernel needs it)
    int grid_cap;           // largest grid the launcher may use (0: the co-resident maximum)
    // work-balanced block ranges (batched step solves): [0] = the grid they
    // were computed for, [1 + b] = first tile of block b, [1 + grid] = end;
    // used when [0] equals the launch's grid, else the uniform ranges
    const int* balance;
    // even-odd solve of a single mixed system (the step's chi = (D^dag)^-1 eta):
    // the systems' compact views and their tile table, given by the caller
    // (null: not available); launch_cg takes the even-odd kernel when the
    // lattice qualifies
    SysDev* sys_eo;
    const int2* eo_tiles;
    int eo_tile_begin, eo_tile_end;
    // every system's compact lattice is tiled by 32 x 16 patches (Nt a multiple
    // of 32, Nx / 2 of 16): batches may take the patch kernel (cg_eop_kernel)
    int eo_patches;
    // inside an even-odd launch: a.sys are the compact views, sys_full the
    // systems' full records (eta, sigma, t64); the first stopping threshold is
    // relative to |eta|^2, tile partial slot 5 of round 0
    const SysDev* sys_full;
    int eo;
};

// Per-chain device record of the Langevin step.
struct ChainDev {
    int Nt, Nx, V;
    int n_rhs;
    int sys0;            // first CG system of the chain
    int tile0, ntiles;   // site tiles of the chain (force / update kernels)
    double m2, lambda, g, m0, r, cut, eps_bar, fixed_dt;
    double lambda6;      // lambda / 6 (divided once on the host: the same IEEE quotient)
    int drift_mode;
    int filter;          // 1 if the cutoff removes modes (FFT path), 0 if white
    uint64_t seed;
    uint32_t chain_id;
    double* phi;
    double* drift;
    double* xi;
    double* white;
    double2* spec;       // Nt*Nx complex work buffer of the noise FFT
    const uint8_t* keep; // Nt*Nx keep-flags of the momentum cutoff
    const double2* tw_t; // twiddles exp(-2 pi i k / Nt), k < Nt
    const double2* tw_x; // twiddles exp(-2 pi i k / Nx), k < Nx
    int64_t step;        // Philox step counter (advanced by the update kernel)
    double time;         // accumulated Langevin time
    yk_obs obs;          // last-step observables
    unsigned counter;    // finaliser counter of the update kernel
    unsigned counter2;
    unsigned long long dmax_bits;   // max |drift| of the step as IEEE bits (atomic max; reset by the update)
    int status;
    // per-step <sigma> = sum sigma / V appended by the update kernels while
    // series_n < series_cap (series null: not recording)
    double* series;
    int64_t series_cap, series_n;
};

struct StepArgs {
    ChainDev* ch;
    int nch;
    const int2* tiles;   // (chain, first site)
    int ntiles;
    int tile_base;       // index of tiles[0] in the per-tile arrays
    double* tile_max;    // per-tile max |drift|
    double2* tile_sum;   // per-tile partial sums
    double* tile_sum2;
};

// Block tables of the coloured-noise passes (built once per context).
struct NoiseTables {
    const int2* rows;    // (chain, t), t even: the row pairs of every chain whose cutoff removes modes
    int nrows;
    const int2* cols;    // (chain, first column) strips of width noise_strip(Nt)
    int ncols;
    const int2* white;   // (chain, first site) tiles of chains with every mode kept
    int nwhite;
};

// Columns per block of the column pass: kBlock / Nt, so that at Nt = 256 each
// block transforms one column.  The FP64 transforms (issued at 1/64 of the
// FP32 rate on GB300) are bound by the FP64 pipe of each SM, so the column
// pass wants as many blocks as there are kept columns rather than busy
// threads (half the block holds a butterfly at Nt = 256).
YK_HD inline int noise_strip(int Nt)
{
    int cw = kBlock / Nt;
    if (cw > 64) cw = 64;
    if (cw < 1) cw = 1;
    return cw;
}

}  // namespace yk
