// yk_api.cu -- the context runtime behind include/yukawa.h.
//
// A context owns every chain's device buffers in one allocation, the device
// tables that let each kernel serve all chains at once (CG systems and tiles,
// site tiles, noise block tables), and the captured CUDA graph of one
// Langevin step.  The reference's equivalents are process-global
// __constant__ parameters (code/src/main.cu:268-278) and per-object managed
// buffers with a device synchronisation after every launch.
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <cstddef>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "yk_host.h"
#include "yk_kernels.h"

using namespace yk;

#define YK_CK(call)                                                                          \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            set_error("%s failed: %s", #call, cudaGetErrorString(e_));                      \
            return YK_ECUDA;                                                                 \
        }                                                                                    \
    } while (0)

namespace {

// Bump allocator over one device allocation.
struct Arena {
    char* base = nullptr;
    size_t size = 0, used = 0;
    size_t reserve(size_t bytes)
    {
        const size_t off = (used + 255) & ~(size_t)255;
        used = off + bytes;
        return off;
    }
    template <typename T>
    T* at(size_t off)
    {
        return reinterpret_cast<T*>(base + off);
    }
};

// Complex (K = 2) workspace of one chain for operator-level calls with
// caller-provided complex buffers.
struct Workspace {
    bool ready = false;
    int R = 0;                  // systems
    void* mem = nullptr;
    SysDev* d_sys = nullptr;
    int2* d_tiles = nullptr;
    CGState* d_state = nullptr;
    Partial* d_partial = nullptr;
    CGCoef* d_coef = nullptr;
    ChainDev* d_chain = nullptr;   // chain copy whose sys0 = 0 refers to d_sys
    int2* d_site_tiles = nullptr;
    std::vector<SysDev> h_sys;
    double* point = nullptr;    // point source (K = 2)
    double* work = nullptr;     // K = 2 spinor scratch
    double* corr = nullptr;     // Nt
};

struct Chain {
    yk_params p;
    yk_action a;
    int Nt, Nx, V;
    int filter;
    int n_rhs_step;             // CG systems per step (0 when g == 0)
    int sys0 = 0, cg_tile0 = 0, cg_tile1 = 0;
    int site_tile0 = 0, nsite_tiles = 0;
    int row0 = 0, nrows = 0, col0 = 0, ncols = 0, white0 = 0, nwhite = 0;
    double *phi, *drift, *xi, *force, *slices;
    double2* spec;
    uint8_t* keep;
    double2 *tw_t, *tw_x;
    Workspace ws;
    LearnedNet* net = nullptr;   // the learned preconditioner (yk_net_setup)
    LearnedNet* pcg_ws = nullptr;   // solver buffers of identity-preconditioned solves without a network
    // pion extension (params.pions): the fields pi_1..3 (3V), their coloured
    // and white noise (3V each), the four forces (4V), the pions' drift (3V),
    // the step's complex sources (n_rhs_pion x 8V) and per-tile sums
    double* series = nullptr;    // recorded per-step <sigma> (yk_series_record)
    int64_t series_cap = 0;
    bool pions = false;
    int n_rhs_pion = 0;          // complex systems per step (0 when g == 0)
    double *pi = nullptr, *pi_xi = nullptr, *pi_white = nullptr, *pforce = nullptr, *pdrift = nullptr;
    double *peta = nullptr, *ptile = nullptr, *ptile_f = nullptr;
};

}  // namespace

struct yk_ctx {
    int dev = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // the step's noise runs on `aux` beside the CG when the CG leaves SMs free
    cudaStream_t aux = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr, join2_ev = nullptr;
    int n_sm = 0;
    bool noise_overlap = true;   // YK_NOISE_OVERLAP=0 at context creation: never
    int overlap_choice = -1;     // the autotuner's choice (1 beside the CG, 0 after it; -1 untuned: beside)
    std::vector<Chain> ch;
    void* mem = nullptr;
    // step tables
    ChainDev* d_chains = nullptr;
    std::vector<ChainDev> h_chains;
    SysDev* d_sys = nullptr;
    int nsys = 0;
    int2* d_sys_tiles = nullptr;
    int n_sys_tiles = 0;
    CGState* d_state = nullptr;
    Partial* d_partial = nullptr;
    CGCoef* d_coef = nullptr;
    unsigned* d_flags = nullptr;   // neighbour flags of the CG launches (shared: one stream)
    GridBarrier* d_bar = nullptr;
    int* d_err = nullptr;
    int* d_nactive = nullptr;
    int* d_anyru = nullptr;
    int* d_balance = nullptr;      // work-balanced block ranges of the batched step CG (CGArgs::balance)
    int2* d_site_tiles = nullptr;
    int n_site_tiles = 0;
    double* d_tile_max = nullptr;
    double2* d_tile_sum = nullptr;
    double* d_tile_sum2 = nullptr;
    int2 *d_rows = nullptr, *d_cols = nullptr, *d_white = nullptr;
    int nrows = 0, ncols = 0, nwhite = 0;
    int max_nx = 1, max_cols = 1;
    // solver settings (shared by all chains of a context)
    int precision = YK_FP64, tol_mode = YK_TOL_ABS, max_iter = 1000, reliable_every = 0;
    double reliable_delta = 0.001;
    double tol = 1e-8;
    // step graph
    cudaGraphExec_t gexec = nullptr;
    bool graph_failed = false;
    // yk_langevin_step_io with pinned host fields: the upload, the step, the
    // downloads of the field, the observables and the error word as one
    // graph per (chain, field pointers), the last few kept
    struct IoGraph {
        int c;
        const double* in;
        double* out;
        const void *in_dev, *out_dev;   // their mapped device addresses when captured
        cudaGraphExec_t exec;
        uint64_t used;
    };
    std::vector<IoGraph> io;
    uint64_t io_clock = 0;
    bool io_failed = false;
    void* io_pin = nullptr;   // pinned staging: the observables, then the error word
    // the transfers as kernels on the mapped host buffers (YK_IO_KERNEL=0 at
    // context creation: copy-engine copies)
    bool io_kernel = true;
    int cg_grid = 0;
    int cg_kernel = 0;   // kernel of the last step CG launch (yk_profile.cg_kernel)
    // mixed precision with every step system fitting one 16-CTA cluster and
    // YK_CG_CLUSTER=1 in the environment: the cluster-resident CG instead of
    // the grid-wide kernel
    bool cg_cluster = false;
    int cluster_sites = 0;   // largest per-CTA share of the step systems
    // single-system mixed solves may take the halo CG kernel (YK_CG_HALO=0 in
    // the environment at context creation: never)
    bool cg_halo = true;
    // the autotuner: grid cap of the step's batched CG (0: the co-resident
    // maximum), chosen by timing candidates before the step graph is captured
    // (YK_AUTOTUNE=0 at context creation: never automatically)
    int cg_grid_cap = 0;
    bool autotune = true, tuned = false;
    // batched step CG: block ranges balanced by the previous step's
    // iterations (YK_CG_BALANCE=1 at context creation; default uniform
    // ranges, which measured faster on the 64-chain configuration)
    bool cg_balance = false;
    yk_tune_result tune = {};
    // profiling: CUDA events around each kernel class of the step
    bool profiling = false;
    struct Rec {
        int cls;
        cudaEvent_t a, b;
    };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    int prof_steps = 0, prof_launches = 0;
    std::vector<int64_t> prof_iters0;
    // pion extension: every chain carries pions; the chains' pion buffers and,
    // per pion field a, a copy of every chain record whose xi is that field's
    // noise (d_pchains[a * n_chains + c]) for the FFT passes
    bool pions = false;
    void* pion_mem = nullptr;
    ChainDev* d_pchains = nullptr;
    // even-odd solves of the step (single mixed system on an even lattice;
    // YK_CG_EO=0 at context creation: never): the systems' compact views and
    // their tile table (the same tile ids as the full table, fewer of them)
    bool cg_eo = false;
    void* eo_mem = nullptr;
    SysDev* d_sys_eo = nullptr;
    int2* d_eo_tiles = nullptr;
    int eo_tile_begin = 0, eo_tile_end = 0;
    bool eo_patches = false;   // every system tiled by 32 x 16 patches of its compact lattice
};

namespace {

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// First columns of the column-pass strips (width cw) that hold a column
// keeping some mode; a column kx keeps some mode exactly when it keeps (0, kx).
std::vector<int> kept_strips(int Nt, int Nx, double cut_fraction, int cw)
{
    std::vector<uint8_t> keep;
    momentum_keep(Nt, Nx, cut_fraction, keep);
    std::vector<int> out;
    for (int x0 = 0; x0 < Nx; x0 += cw) {
        bool any = false;
        for (int x = x0; x < x0 + cw && x < Nx; ++x) any = any || keep[x];
        if (any) out.push_back(x0);
    }
    return out;
}

int check_params(const yk_params& p, int c)
{
    if (p.Nt < 2 || p.Nx < 2) {
        set_error("chain %d: lattice %dx%d too small (need Nt, Nx >= 2)", c, p.Nt, p.Nx);
        return YK_EINVAL;
    }
    if ((int64_t)p.Nt * p.Nx > (1LL << 27)) {
        set_error("chain %d: lattice %dx%d too large", c, p.Nt, p.Nx);
        return YK_EINVAL;
    }
    if (!all_modes_kept(p.Nt, p.Nx, p.cut_fraction)) {
        const bool okt = (is_pow2(p.Nt) && p.Nt <= kMaxFFT) || p.Nt <= kMaxDFT;
        const bool okx = (is_pow2(p.Nx) && p.Nx <= kMaxFFT) || p.Nx <= kMaxDFT;
        if (!okt || !okx) {
            set_error("chain %d: coloured noise needs Nt, Nx powers of two <= %d or <= %d (got %dx%d)", c,
                      kMaxFFT, kMaxDFT, p.Nt, p.Nx);
            return YK_EINVAL;
        }
    }
    if (p.n_rhs < 1 || p.n_rhs > 64) {
        set_error("chain %d: n_rhs = %d outside [1, 64]", c, p.n_rhs);
        return YK_EINVAL;
    }
    if (p.precision != YK_FP64 && p.precision != YK_MIXED) {
        set_error("chain %d: precision must be YK_FP64 or YK_MIXED", c);
        return YK_EINVAL;
    }
    if (p.cg_max_iter < 0 || p.cg_max_iter > 1000000) {
        set_error("chain %d: cg_max_iter out of range", c);
        return YK_EINVAL;
    }
    if (p.reliable_every < 0 || !(p.reliable_delta > 0.0 && p.reliable_delta < 1.0)) {
        set_error("chain %d: reliable_every must be >= 0 and reliable_delta in (0, 1)", c);
        return YK_EINVAL;
    }
    if (p.pions != 0 && p.pions != 1) {
        set_error("chain %d: pions must be 0 or 1", c);
        return YK_EINVAL;
    }
    return YK_OK;
}

// Calls that act on the real sigma-only operator refuse contexts with pions.
int no_pions(const yk_ctx* ctx, const char* what)
{
    if (ctx && ctx->pions) {
        set_error("%s: not available with pions (it acts on the real sigma-only operator)", what);
        return YK_EINVAL;
    }
    return YK_OK;
}

int ntiles_of(int V) { return (V + kTile - 1) / kTile; }

int chain_ok(const yk_ctx* ctx, int c)
{
    if (!ctx || c < 0 || c >= (int)ctx->ch.size()) {
        set_error("invalid context or chain index %d", c);
        return YK_EINVAL;
    }
    return YK_OK;
}

int status_of_err(yk_ctx* ctx)
{
    int e = 0;
    YK_CK(cudaMemcpyAsync(&e, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    if (e) {
        set_error("a bounded device wait gave up (status %d)", e);
        return YK_ETIMEOUT;
    }
    return YK_OK;
}

CGArgs base_args(yk_ctx* ctx)
{
    CGArgs a = {};
    a.bar = ctx->d_bar;
    a.flags = ctx->d_flags;
    a.err = ctx->d_err;
    a.n_active = ctx->d_nactive;
    a.any_ru = ctx->d_anyru;
    a.max_iter = ctx->max_iter;
    a.tol_mode = ctx->tol_mode;
    a.tol = ctx->tol;
    a.reliable_every = ctx->reliable_every;
    a.reliable_delta = ctx->reliable_delta;
    a.mtype = YK_DAGGER;
    a.grid_cap = ctx->cg_grid_cap;
    return a;
}

StepArgs step_args(yk_ctx* ctx)
{
    StepArgs s = {};
    s.ch = ctx->d_chains;
    s.nch = (int)ctx->ch.size();
    s.tiles = ctx->d_site_tiles;
    s.ntiles = ctx->n_site_tiles;
    s.tile_max = ctx->d_tile_max;
    s.tile_sum = ctx->d_tile_sum;
    s.tile_sum2 = ctx->d_tile_sum2;
    return s;
}

cudaEvent_t take_event(yk_ctx* ctx)
{
    if (!ctx->pool.empty()) {
        cudaEvent_t e = ctx->pool.back();
        ctx->pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Events around one kernel class when profiling (no-ops otherwise).
void prof_begin(yk_ctx* ctx, cudaEvent_t* a)
{
    if (!ctx->profiling) return;
    *a = take_event(ctx);
    cudaEventRecord(*a, ctx->stream);
}

void prof_end(yk_ctx* ctx, int cls, cudaEvent_t a, int launches)
{
    if (!ctx->profiling) return;
    cudaEvent_t b = take_event(ctx);
    cudaEventRecord(b, ctx->stream);
    ctx->recs.push_back({cls, a, b});
    ctx->prof_launches += launches;
}

// Enqueues one Langevin step of every chain.  The coloured noise does not
// depend on the step's CG: when the persistent CG (one block per SM) leaves
// SMs free, the noise passes run on the auxiliary stream beside it, on at
// most that many blocks, and the update waits for them.  Profiled steps run
// the kernel classes one after the other.
void eo_args(const yk_ctx* ctx, CGArgs& a);

// The arguments of the step's CG launch (every system, Philox sources).
CGArgs step_cg_args(yk_ctx* ctx)
{
    CGArgs a = base_args(ctx);
    a.sys = ctx->d_sys;
    a.sys_first = 0;
    a.sys_count = ctx->nsys;
    a.tiles = ctx->d_sys_tiles;
    a.tile_begin = 0;
    a.tile_end = ctx->n_sys_tiles;
    a.eta_kind = 2;
    a.st = ctx->d_state;
    a.partial = ctx->d_partial;
    a.coef = ctx->d_coef;
    if (ctx->nsys == 1 && ctx->cg_halo)
        for (const Chain& C : ctx->ch)
            if (C.n_rhs_step > 0) {
                a.solo_nt = C.Nt;
                a.solo_nx = C.Nx;
            }
    eo_args(ctx, a);
    return a;
}

int enqueue_step(yk_ctx* ctx)
{
    cudaEvent_t e = nullptr;
    NoiseTables nt = {ctx->d_rows, ctx->nrows, ctx->d_cols, ctx->ncols, ctx->d_white, ctx->nwhite};
    int free_sm = 0;
    if (ctx->noise_overlap && !ctx->profiling && !ctx->cg_cluster && ctx->nsys > 0 && ctx->nrows > 0)
        free_sm = ctx->n_sm - cg_predict_grid(step_cg_args(ctx), ctx->precision == YK_MIXED);
    const bool overlap = free_sm >= 8 && ctx->overlap_choice != 0;
    if (overlap) {
        YK_CK(cudaEventRecord(ctx->fork_ev, ctx->stream));
        YK_CK(cudaStreamWaitEvent(ctx->aux, ctx->fork_ev, 0));
        YK_CK(launch_noise_tables(ctx->d_chains, nt, ctx->max_nx, ctx->max_cols, nullptr, ctx->aux, free_sm));
        YK_CK(cudaEventRecord(ctx->join_ev, ctx->aux));
        // the next step's sources, which its CG would otherwise generate first
        YK_CK(launch_eta_ahead(ctx->d_sys, ctx->d_sys_tiles, ctx->n_sys_tiles, free_sm, ctx->aux));
        YK_CK(cudaEventRecord(ctx->join2_ev, ctx->aux));
    } else {
        prof_begin(ctx, &e);
        YK_CK(launch_noise_tables(ctx->d_chains, nt, ctx->max_nx, ctx->max_cols, nullptr, ctx->stream));
        prof_end(ctx, 0, e, (ctx->nwhite > 0 ? 1 : 0) + (ctx->nrows > 0 ? 3 : 0));
    }
    if (ctx->nsys > 0) {
        prof_begin(ctx, &e);
        CGArgs a = step_cg_args(ctx);
        if (ctx->cg_cluster) {
            YK_CK(launch_eta(ctx->d_sys, ctx->d_sys_tiles, ctx->n_sys_tiles, 2, ctx->stream));
            YK_CK(launch_cg_cluster(a, ctx->cluster_sites, ctx->stream));
            ctx->cg_grid = 16 * ctx->nsys;
            ctx->cg_kernel = 2;
            prof_end(ctx, 1, e, 2);
        } else {
            // batched: block ranges balanced by the previous step's iterations
            const bool bal = ctx->nsys > 1 && ctx->cg_balance && !ctx->cg_eo;
            if (bal) a.balance = ctx->d_balance;
            YK_CK(launch_cg(a, 1, ctx->precision == YK_MIXED, ctx->stream, &ctx->cg_grid, &ctx->cg_kernel));
            if (bal) YK_CK(launch_cg_balance(a, ctx->cg_grid, ctx->d_balance, ctx->stream));
            prof_end(ctx, 1, e, bal ? 3 : 2);
        }
    }
    StepArgs s = step_args(ctx);
    prof_begin(ctx, &e);
    YK_CK(launch_force_drift(s, ctx->d_sys, 0, 1, ctx->stream, ctx->d_state));
    prof_end(ctx, 2, e, 1);
    if (overlap) {
        YK_CK(cudaStreamWaitEvent(ctx->stream, ctx->join_ev, 0));   // xi of this step
        // the next step's eta: its kernel reads the chain's step counter, which
        // the update advances, so it must be done before the update runs
        YK_CK(cudaStreamWaitEvent(ctx->stream, ctx->join2_ev, 0));
    }
    prof_begin(ctx, &e);
    YK_CK(launch_update(s, ctx->d_state, ctx->stream));
    prof_end(ctx, 3, e, 1);
    if (ctx->profiling) ctx->prof_steps += 1;
    return YK_OK;
}

// Complex (K = 2) workspace with R systems for chain c.
int ensure_ws(yk_ctx* ctx, int c, int R)
{
    Chain& C = ctx->ch[c];
    Workspace& w = C.ws;
    if (w.ready && w.R >= R) return YK_OK;
    if (w.mem) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(w.mem);
        w = Workspace();
    }
    const int V = C.V, nt = ntiles_of(V);
    const size_t v64 = sizeof(double) * 8 * (size_t)V, v32 = sizeof(float) * 8 * (size_t)V;
    Arena ar;
    const size_t o_sys = ar.reserve(sizeof(SysDev) * R);
    const size_t o_tiles = ar.reserve(sizeof(int2) * (size_t)R * nt);
    const size_t o_state = ar.reserve(sizeof(CGState) * R);
    const size_t o_part = ar.reserve(sizeof(Partial) * (size_t)R * nt);
    const size_t o_coef = ar.reserve(sizeof(CGCoef) * R);
    const size_t o_chain = ar.reserve(sizeof(ChainDev));
    const size_t o_stile = ar.reserve(sizeof(int2) * nt);
    const size_t o_point = ar.reserve(v64);
    const size_t o_work = ar.reserve(v64);
    const size_t o_corr = ar.reserve(sizeof(double) * C.Nt);
    constexpr int NVEC = 15;   // FP64: x r0 r1 p0 p1 t Ap; FP32: r0 r1 p0 p1 t Ap xs; diag
    std::vector<size_t> o_vec(R * NVEC);
    for (int j = 0; j < R; ++j) {
        for (int q = 0; q < 7; ++q) o_vec[j * NVEC + q] = ar.reserve(v64);
        for (int q = 7; q < 14; ++q) o_vec[j * NVEC + q] = ar.reserve(v32);
        o_vec[j * NVEC + 14] = ar.reserve(sizeof(float) * (size_t)V);
    }
    void* mem = nullptr;
    if (cudaMalloc(&mem, ar.used) != cudaSuccess) {
        cudaGetLastError();
        set_error("workspace allocation of %zu bytes failed", ar.used);
        return YK_ENOMEM;
    }
    ar.base = (char*)mem;
    w.mem = mem;
    w.R = R;
    w.d_sys = ar.at<SysDev>(o_sys);
    w.d_tiles = ar.at<int2>(o_tiles);
    w.d_state = ar.at<CGState>(o_state);
    w.d_partial = ar.at<Partial>(o_part);
    w.d_coef = ar.at<CGCoef>(o_coef);
    w.d_chain = ar.at<ChainDev>(o_chain);
    w.d_site_tiles = ar.at<int2>(o_stile);
    w.point = ar.at<double>(o_point);
    w.work = ar.at<double>(o_work);
    w.corr = ar.at<double>(o_corr);
    w.h_sys.assign(R, SysDev());
    std::vector<int2> tiles((size_t)R * nt);
    for (int j = 0; j < R; ++j) {
        SysDev& S = w.h_sys[j];
        std::memset(&S, 0, sizeof(S));
        S.chain = c;
        S.rhs = j;
        S.Nt = C.Nt;
        S.Nx = C.Nx;
        S.V = V;
        S.tile0 = j * nt;
        S.ntiles = nt;
        S.m0 = C.a.m0;
        S.g = C.a.g;
        S.r = C.a.r;
        S.sigma = C.phi;
        S.pi = C.pions ? C.pi : nullptr;
        const size_t* o = &o_vec[(size_t)j * NVEC];
        S.x = ar.at<double>(o[0]);
        S.r64[0] = ar.at<double>(o[1]);
        S.r64[1] = ar.at<double>(o[2]);
        S.p64[0] = ar.at<double>(o[3]);
        S.p64[1] = ar.at<double>(o[4]);
        S.t64 = ar.at<double>(o[5]);
        S.Ap64 = ar.at<double>(o[6]);
        S.r32[0] = ar.at<float>(o[7]);
        S.r32[1] = ar.at<float>(o[8]);
        S.p32[0] = ar.at<float>(o[9]);
        S.p32[1] = ar.at<float>(o[10]);
        S.t32 = ar.at<float>(o[11]);
        S.Ap32 = ar.at<float>(o[12]);
        S.xs32 = ar.at<float>(o[13]);
        S.diag32 = ar.at<float>(o[14]);
        S.gen_eta = 0;
        for (int t = 0; t < nt; ++t) tiles[(size_t)j * nt + t] = make_int2(j, t * kTile);
    }
    std::vector<int2> stiles(nt);
    for (int t = 0; t < nt; ++t) stiles[t] = make_int2(0, t * kTile);
    YK_CK(cudaMemcpyAsync(w.d_tiles, tiles.data(), sizeof(int2) * tiles.size(), cudaMemcpyHostToDevice,
                          ctx->stream));
    YK_CK(cudaMemcpyAsync(w.d_site_tiles, stiles.data(), sizeof(int2) * nt, cudaMemcpyHostToDevice,
                          ctx->stream));
    YK_CK(cudaMemsetAsync(w.d_state, 0, sizeof(CGState) * R, ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    w.ready = true;
    return YK_OK;
}

// Solves the first `count` systems of chain c's complex workspace.
int ws_solve(yk_ctx* ctx, int c, int count, int mtype, double tol, int tol_mode, int max_iter, int precision,
             yk_solve_stats* stats)
{
    Chain& C = ctx->ch[c];
    Workspace& w = C.ws;
    YK_CK(cudaMemcpyAsync(w.d_sys, w.h_sys.data(), sizeof(SysDev) * count, cudaMemcpyHostToDevice, ctx->stream));
    CGArgs a = base_args(ctx);
    a.sys = w.d_sys;
    a.sys_first = 0;
    a.sys_count = count;
    a.tiles = w.d_tiles;
    a.tile_begin = 0;
    a.tile_end = count * ntiles_of(C.V);
    a.eta_kind = 0;
    a.st = w.d_state;
    a.partial = w.d_partial;
    a.coef = w.d_coef;
    a.mtype = mtype;
    a.tol = tol;
    a.tol_mode = tol_mode;
    a.max_iter = max_iter;
    YK_CK(launch_cg(a, 2, precision == YK_MIXED, ctx->stream, nullptr));
    std::vector<CGState> st(count);
    YK_CK(cudaMemcpyAsync(st.data(), w.d_state, sizeof(CGState) * count, cudaMemcpyDeviceToHost, ctx->stream));
    int rc = status_of_err(ctx);
    if (rc) return rc;
    yk_solve_stats s = {};
    s.converged = 1;
    int status = 0;
    for (int j = 0; j < count; ++j) {
        s.iterations += st[j].iters;
        s.reliable_updates += st[j].n_ru;
        s.rr += st[j].rr;
        s.rr0 += st[j].rr0;
        if (!st[j].converged) s.converged = 0;
        if (!status && st[j].status) status = st[j].status;
    }
    if (stats) *stats = s;
    if (status) {
        set_error("CG: status %d after %d iterations (|r|^2 = %g)", status, s.iterations, s.rr);
        return status;
    }
    return YK_OK;
}

// Runs the CG of chain c's step systems (K = 1) with Philox right-hand sides
// of stream `kind` at the chain's current step.
// want_x: the caller reads x (the solution of D^dag D x = b); otherwise the
// step's even-odd solve may run, which leaves chi = D x in t64 instead.
int chain_solve(yk_ctx* ctx, int c, int kind, yk_solve_stats* stats, bool want_x = false)
{
    Chain& C = ctx->ch[c];
    if (C.n_rhs_step == 0) {
        if (stats) *stats = yk_solve_stats{0, 0, 0.0, 0.0, 1};
        return YK_OK;
    }
    CGArgs a = base_args(ctx);
    a.sys = ctx->d_sys;
    a.sys_first = C.sys0;
    a.sys_count = C.n_rhs_step;
    a.tiles = ctx->d_sys_tiles;
    a.tile_begin = C.cg_tile0;
    a.tile_end = C.cg_tile1;
    a.eta_kind = kind;
    a.st = ctx->d_state;
    a.partial = ctx->d_partial;
    a.coef = ctx->d_coef;
    if (C.n_rhs_step == 1 && ctx->cg_halo) {
        a.solo_nt = C.Nt;
        a.solo_nx = C.Nx;
    }
    if (!want_x) eo_args(ctx, a);
    if (ctx->cg_cluster) {
        YK_CK(launch_eta(ctx->d_sys, ctx->d_sys_tiles + C.cg_tile0, C.cg_tile1 - C.cg_tile0, kind, ctx->stream));
        YK_CK(launch_cg_cluster(a, ctx->cluster_sites, ctx->stream));
    } else {
        YK_CK(launch_cg(a, 1, ctx->precision == YK_MIXED, ctx->stream, nullptr));
    }
    std::vector<CGState> st(C.n_rhs_step);
    YK_CK(cudaMemcpyAsync(st.data(), ctx->d_state + C.sys0, sizeof(CGState) * C.n_rhs_step,
                          cudaMemcpyDeviceToHost, ctx->stream));
    int rc = status_of_err(ctx);
    if (rc) return rc;
    yk_solve_stats s = {};
    s.converged = 1;
    int status = 0;
    for (auto& q : st) {
        s.iterations += q.iters;
        s.reliable_updates += q.n_ru;
        s.rr += q.rr;
        s.rr0 += q.rr0;
        if (!q.converged) s.converged = 0;
        if (!status && q.status) status = q.status;
    }
    if (stats) *stats = s;
    if (status) {
        set_error("CG: status %d after %d iterations", status, s.iterations);
        return status;
    }
    return YK_OK;
}

// Where the step's coloured noise and the next step's sources run: beside the
// CG on an auxiliary stream (the SMs its grid leaves free) or after it on the
// main stream.  A short solve finishes before the auxiliary work on the few
// free SMs, and the update then waits for it.  Both forms are timed over two
// steps after one warm-up step, each from the chains' state saved here and
// restored after (fields and chain records; the steps are deterministic, so
// tuning changes no result).
int tune_overlap(yk_ctx* ctx)
{
    yk_tune_result& T = ctx->tune;
    if (!ctx->noise_overlap || ctx->cg_cluster || ctx->nsys == 0 || ctx->nrows == 0 || ctx->pions) return YK_OK;
    if (ctx->n_sm - cg_predict_grid(step_cg_args(ctx), ctx->precision == YK_MIXED) < 8) return YK_OK;
    const int nch = (int)ctx->ch.size();
    size_t nphi = 0;
    for (const Chain& C : ctx->ch) nphi += (size_t)C.V;
    void* save = nullptr;
    if (cudaMalloc(&save, sizeof(double) * nphi + sizeof(ChainDev) * nch) != cudaSuccess) {
        cudaGetLastError();
        return YK_OK;   // no room to save the state: keep the untuned form
    }
    double* sphi = static_cast<double*>(save);
    ChainDev* sch = reinterpret_cast<ChainDev*>(sphi + nphi);
    auto copy_state = [&](bool to_save) -> cudaError_t {
        size_t off = 0;
        cudaError_t e = cudaSuccess;
        for (const Chain& C : ctx->ch) {
            e = to_save ? cudaMemcpyAsync(sphi + off, C.phi, sizeof(double) * C.V, cudaMemcpyDeviceToDevice, ctx->stream)
                        : cudaMemcpyAsync(C.phi, sphi + off, sizeof(double) * C.V, cudaMemcpyDeviceToDevice, ctx->stream);
            if (e != cudaSuccess) return e;
            off += C.V;
        }
        return to_save ? cudaMemcpyAsync(sch, ctx->d_chains, sizeof(ChainDev) * nch, cudaMemcpyDeviceToDevice, ctx->stream)
                       : cudaMemcpyAsync(ctx->d_chains, sch, sizeof(ChainDev) * nch, cudaMemcpyDeviceToDevice, ctx->stream);
    };
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = YK_OK;
    float ms[2] = {0.f, 0.f};
    const bool profiling = ctx->profiling;   // the tuning steps are not profiled steps
    ctx->profiling = false;
    cudaError_t e = copy_state(true);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    for (int cand = 1; cand >= 0 && e == cudaSuccess && rc == YK_OK; --cand) {
        ctx->overlap_choice = cand;
        rc = enqueue_step(ctx);
        if (rc == YK_OK) e = cudaEventRecord(e0, ctx->stream);
        for (int rep = 0; rep < 2 && rc == YK_OK && e == cudaSuccess; ++rep) rc = enqueue_step(ctx);
        if (rc == YK_OK && e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
        if (rc == YK_OK && e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (rc == YK_OK && e == cudaSuccess) e = cudaEventElapsedTime(&ms[cand], e0, e1);
        if (rc == YK_OK && e == cudaSuccess) rc = status_of_err(ctx);
        if (rc == YK_OK && e == cudaSuccess) e = copy_state(false);
    }
    ctx->profiling = profiling;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(save);
    if (rc) return rc;
    if (e != cudaSuccess) {
        set_error("autotune (noise placement): %s", cudaGetErrorString(e));
        return YK_ECUDA;
    }
    ctx->overlap_choice = ms[1] <= ms[0] ? 1 : 0;
    T.noise_overlap = ctx->overlap_choice;
    T.step_ms_overlap = ms[1] / 2.f;
    T.step_ms_serial = ms[0] / 2.f;
    return YK_OK;
}

// The autotuner.  Batched steps (several CG systems in one launch): the grid
// of the persistent CG (the batched even-odd kernel's, or how many tiles
// each block of cg_kernel owns), by timing the
// step's CG (sources of Philox kind 100, which no step draws; 48 iterations;
// two launches after one warm-up) at each candidate: the co-resident maximum,
// 3/4 and 1/2 of it, one block per SM and half of that.  Fewer blocks own
// more tiles each and synchronise fewer arrivals; more blocks hide latency.
// The iterates do not depend on the grid (tile partials are summed in a fixed
// order), so tuning never changes results.  The learned solver's convolution
// tile is tuned by the network itself on its first solve (net_tile reports it).
int run_autotune(yk_ctx* ctx)
{
    yk_tune_result& T = ctx->tune;
    T = yk_tune_result{};
    const bool mixed = ctx->precision == YK_MIXED;
    if (ctx->nsys > 1 && !ctx->cg_cluster) {
        const int maxg = ctx->cg_eo ? cg_eob_max_grid() : cg_max_grid(1, mixed);
        std::vector<int> cand = {maxg, maxg * 3 / 4, maxg / 2, ctx->n_sm, ctx->n_sm / 2};
        std::sort(cand.begin(), cand.end(), std::greater<int>());
        cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        YK_CK(cudaEventCreate(&e0));
        YK_CK(cudaEventCreate(&e1));
        CGArgs a = base_args(ctx);
        a.sys = ctx->d_sys;
        a.sys_first = 0;
        a.sys_count = ctx->nsys;
        a.tiles = ctx->d_sys_tiles;
        a.tile_begin = 0;
        a.tile_end = ctx->n_sys_tiles;
        a.eta_kind = 100;
        a.st = ctx->d_state;
        a.partial = ctx->d_partial;
        a.coef = ctx->d_coef;
        eo_args(ctx, a);   // the kernel the step runs
        a.max_iter = std::min(ctx->max_iter, 48);
        int best = 0;
        float best_ms = 0.f;
        for (int c : cand) {
            if (c < 8 || c > maxg) continue;
            if ((ctx->n_sys_tiles + c - 1) / c > kMaxTilesPerBlock) continue;
            a.grid_cap = c;
            cudaError_t e = launch_cg(a, 1, mixed, ctx->stream, nullptr);
            if (e == cudaSuccess) e = cudaEventRecord(e0, ctx->stream);
            for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) e = launch_cg(a, 1, mixed, ctx->stream, nullptr);
            if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (e != cudaSuccess) {
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                set_error("autotune: %s", cudaGetErrorString(e));
                return YK_ECUDA;
            }
            if (int rc = status_of_err(ctx)) {
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                return rc;
            }
            ++T.cg_candidates;
            if (c == maxg) T.cg_ms_max = ms;
            if (!best || ms < best_ms) {
                best = c;
                best_ms = ms;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        ctx->cg_grid_cap = best == maxg ? 0 : best;
        T.cg_grid = best;
        T.cg_grid_max = maxg;
        T.cg_ms_chosen = best_ms;
    }
    T.noise_overlap = -1;
    if (int rc = tune_overlap(ctx)) return rc;
    for (const Chain& C : ctx->ch)
        if (C.net) {
            net_tile(C.net, &T.conv_rows, &T.conv_cols, &T.conv_layers_per_launch);
            T.pcg_inner_tol = pcg_inner_choice(C.net);
            break;
        }
    ctx->tuned = true;
    return YK_OK;
}

StepArgs chain_step_args(yk_ctx* ctx, int c)
{
    StepArgs s = step_args(ctx);
    s.tiles = ctx->d_site_tiles + ctx->ch[c].site_tile0;
    s.ntiles = ctx->ch[c].nsite_tiles;
    s.tile_base = ctx->ch[c].site_tile0;
    return s;
}

// ---------------------------------------------------------------- pions
// Buffers of the pion extension (one allocation for every chain), the initial
// pions (iid Uniform[-1, 1] from Philox stream kind 0, rhs a, or zeros for
// YK_INIT_NONE) and the per-field chain records of the noise passes.
int pion_setup(yk_ctx* ctx)
{
    const int nch = (int)ctx->ch.size();
    Arena ar;
    struct POff {
        size_t pi, xi, white, force, drift, eta, tile, tilef;
    };
    std::vector<POff> po(nch);
    const size_t o_pch = ar.reserve(sizeof(ChainDev) * 3 * (size_t)nch);
    for (int c = 0; c < nch; ++c) {
        const Chain& C = ctx->ch[c];
        const size_t V = C.V, nt = ntiles_of(C.V);
        po[c].pi = ar.reserve(8 * 3 * V);
        po[c].xi = ar.reserve(8 * 3 * V);
        po[c].white = ar.reserve(8 * 3 * V);
        po[c].force = ar.reserve(8 * 4 * V);
        po[c].drift = ar.reserve(8 * 3 * V);
        po[c].eta = ar.reserve(8 * 8 * V * (size_t)std::max(C.n_rhs_pion, 1));
        po[c].tile = ar.reserve(8 * 6 * nt);
        po[c].tilef = ar.reserve(8 * nt);
    }
    if (cudaMalloc(&ctx->pion_mem, ar.used) != cudaSuccess) {
        cudaGetLastError();
        set_error("pion allocation of %zu bytes failed", ar.used);
        return YK_ENOMEM;
    }
    ar.base = (char*)ctx->pion_mem;
    YK_CK(cudaMemsetAsync(ctx->pion_mem, 0, ar.used, ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    ctx->d_pchains = ar.at<ChainDev>(o_pch);
    std::vector<ChainDev> pch(3 * (size_t)nch);
    for (int c = 0; c < nch; ++c) {
        Chain& C = ctx->ch[c];
        C.pi = ar.at<double>(po[c].pi);
        C.pi_xi = ar.at<double>(po[c].xi);
        C.pi_white = ar.at<double>(po[c].white);
        C.pforce = ar.at<double>(po[c].force);
        C.pdrift = ar.at<double>(po[c].drift);
        C.peta = ar.at<double>(po[c].eta);
        C.ptile = ar.at<double>(po[c].tile);
        C.ptile_f = ar.at<double>(po[c].tilef);
        std::vector<double> pi(3 * (size_t)C.V, 0.0);
        if (C.p.init != YK_INIT_NONE)
            for (int a = 0; a < 3; ++a)
                philox_uniform_field((uint64_t)C.p.seed, (uint32_t)c, C.V, pi.data() + (size_t)a * C.V,
                                     (uint32_t)(a + 1));
        YK_CK(cudaMemcpy(C.pi, pi.data(), sizeof(double) * pi.size(), cudaMemcpyHostToDevice));
        for (int a = 0; a < 3; ++a) {
            ChainDev H = ctx->h_chains[c];
            H.xi = C.pi_xi + (size_t)a * C.V;
            pch[(size_t)a * nch + c] = H;
        }
    }
    YK_CK(cudaMemcpy(ctx->d_pchains, pch.data(), sizeof(ChainDev) * pch.size(), cudaMemcpyHostToDevice));
    return YK_OK;
}

// Compact (even-odd) views of the step's single mixed system: the lattice of
// one parity class (Nx / 2 columns, V / 2 sites) over the system's buffers --
// the FP32 vectors compact, x = chi_e followed by rhs_e, t64 the full chi at
// the end -- and its tile table.
int eo_setup(yk_ctx* ctx, const std::vector<SysDev>& hs)
{
    // Compact views of the step's systems: a single system (cg_eo_kernel, or
    // cg_eob_kernel when its lattice is too large for the halo kernel's shared
    // memory) or every system of a batched step (cg_eob_kernel).  Mixed
    // precision, sigma-only, every lattice even with Nx >= 4.
    const char* env = getenv("YK_CG_EO");
    if ((env && env[0] == '0') || ctx->nsys < 1 || ctx->nsys > kEobMaxSystems || ctx->precision != YK_MIXED ||
        ctx->cg_cluster || ctx->pions || (ctx->nsys == 1 && !ctx->cg_halo))
        return YK_OK;
    for (const Chain& q : ctx->ch)
        if (q.n_rhs_step > 0 && ((q.Nt & 1) || (q.Nx & 1) || q.Nx < 4)) return YK_OK;
    std::vector<SysDev> views(hs);
    std::vector<int2> tiles(ctx->n_sys_tiles, make_int2(0, 0));
    size_t n_dinv = 0;
    for (int sidx = 0; sidx < ctx->nsys; ++sidx) n_dinv += (size_t)hs[sidx].V / 2;
    const size_t o_tiles = ((sizeof(SysDev) * ctx->nsys + 255) / 256) * 256;
    const size_t o_dinv = o_tiles + ((sizeof(int2) * tiles.size() + 255) / 256) * 256;
    if (cudaMalloc(&ctx->eo_mem, o_dinv + sizeof(double) * n_dinv) != cudaSuccess) {
        cudaGetLastError();
        set_error("even-odd view allocation failed");
        return YK_ENOMEM;
    }
    double* dinv = reinterpret_cast<double*>(static_cast<char*>(ctx->eo_mem) + o_dinv);
    for (int sidx = 0; sidx < ctx->nsys; ++sidx) {
        const SysDev& S = hs[sidx];
        SysDev& E = views[sidx];
        const int Ve = S.V / 2, nte = ntiles_of(Ve);
        E.Nx = S.Nx / 2;
        E.V = Ve;
        E.tile0 = S.tile0;   // the first nte slots of the system's tile range
        E.ntiles = nte;
        E.dinv = dinv;
        dinv += Ve;
        E.v32 = S.xs32 + 4 * (size_t)Ve;     // the halves the compact vectors leave free
        E.w32 = S.r32[1] + 4 * (size_t)Ve;
        for (int t = 0; t < nte; ++t) tiles[S.tile0 + t] = make_int2(sidx, t * kTile);
    }
    ctx->d_sys_eo = reinterpret_cast<SysDev*>(ctx->eo_mem);
    ctx->d_eo_tiles = reinterpret_cast<int2*>(static_cast<char*>(ctx->eo_mem) + o_tiles);
    YK_CK(cudaMemcpy(ctx->d_sys_eo, views.data(), sizeof(SysDev) * views.size(), cudaMemcpyHostToDevice));
    YK_CK(cudaMemcpy(ctx->d_eo_tiles, tiles.data(), sizeof(int2) * tiles.size(), cudaMemcpyHostToDevice));
    if (ctx->nsys == 1) {
        ctx->eo_tile_begin = hs[0].tile0;
        ctx->eo_tile_end = hs[0].tile0 + views[0].ntiles;
    } else {
        ctx->eo_tile_begin = 0;
        ctx->eo_tile_end = ctx->n_sys_tiles;
    }
    // every step system's compact lattice tiled by 32 x 16 patches: batches may
    // take the patch kernel
    ctx->eo_patches = true;
    for (const Chain& q : ctx->ch)
        if (q.n_rhs_step > 0 && ((q.Nt % 32) || ((q.Nx / 2) % 16))) ctx->eo_patches = false;
    ctx->cg_eo = true;
    return YK_OK;
}

// The step CG's even-odd views, when the context has them.
void eo_args(const yk_ctx* ctx, CGArgs& a)
{
    if (!ctx->cg_eo) return;
    a.sys_eo = ctx->d_sys_eo;
    a.eo_tiles = ctx->d_eo_tiles;
    a.eo_tile_begin = ctx->eo_tile_begin;
    a.eo_tile_end = ctx->eo_tile_end;
    a.eo_patches = ctx->eo_patches ? 1 : 0;
}

// The complex systems of a pion chain: sources eta (device, n_rhs x 8V) or,
// when null, Philox stream `kind` at the chain's current step; solved with
// the pion operator on the chain's workspace.
int pion_solve(yk_ctx* ctx, int c, int kind, const double* eta, int precision, yk_solve_stats* stats)
{
    Chain& C = ctx->ch[c];
    const int R = C.n_rhs_pion;
    if (R == 0) {
        if (stats) *stats = yk_solve_stats{0, 0, 0.0, 0.0, 1};
        return YK_OK;
    }
    if (int rc = ensure_ws(ctx, c, R)) return rc;
    Workspace& w = C.ws;
    if (!eta) {
        YK_CK(launch_pion_eta(ctx->d_chains + c, C.peta, R, kind, C.V, ctx->stream));
        eta = C.peta;
    }
    for (int j = 0; j < R; ++j) w.h_sys[j].b = const_cast<double*>(eta) + (size_t)j * 8 * C.V;
    return ws_solve(ctx, c, R, YK_DAGGER, ctx->tol, ctx->tol_mode, ctx->max_iter, precision, stats);
}

// One Langevin step of pion chain c: four coloured noises, the complex solves,
// the four forces, drift and update (yk_pion.cu).  The solves report their
// statistics to the host, so the step is driven from the host (no graph).
int pion_step(yk_ctx* ctx, int c)
{
    Chain& C = ctx->ch[c];
    const int nch = (int)ctx->ch.size();
    const NoiseTables nt = {ctx->d_rows + C.row0, C.nrows, ctx->d_cols + C.col0, C.ncols, ctx->d_white + C.white0,
                            C.nwhite};
    YK_CK(launch_noise_tables(ctx->d_chains, nt, ctx->max_nx, ctx->max_cols, nullptr, ctx->stream));
    YK_CK(launch_pion_white(ctx->d_chains + c, C.pi_white, C.V, ctx->stream));
    for (int a = 0; a < 3; ++a)
        YK_CK(launch_noise_tables(ctx->d_pchains + (size_t)a * nch, nt, ctx->max_nx, ctx->max_cols,
                                  C.pi_white + (size_t)a * C.V, ctx->stream));
    const int rc = pion_solve(ctx, c, 2, nullptr, ctx->precision, nullptr);
    if (rc && rc != YK_ENOCONV) return rc;
    const int R = C.n_rhs_pion;
    YK_CK(launch_pion_force(ctx->d_chains + c, C.ws.d_sys, R, C.pi, C.pforce, C.V, ctx->stream));
    YK_CK(launch_pion_drift_update(ctx->d_chains + c, C.pi, C.pforce, C.pdrift, C.pi_xi, C.ptile, C.ptile_f,
                                   C.ws.d_state, R, C.V, ctx->stream));
    return YK_OK;
}

}  // namespace

extern "C" {

int yk_ctx_create(const yk_params* params, int n_chains, yk_ctx** out)
{
    if (!params || n_chains < 1 || !out) {
        set_error("yk_ctx_create: bad arguments");
        return YK_EINVAL;
    }
    *out = nullptr;
    for (int c = 0; c < n_chains; ++c) {
        int rc = check_params(params[c], c);
        if (rc) return rc;
    }
    const yk_params& p0 = params[0];
    for (int c = 1; c < n_chains; ++c) {
        const yk_params& p = params[c];
        if (p.precision != p0.precision || p.cg_tol_mode != p0.cg_tol_mode || p.cg_tol != p0.cg_tol ||
            p.cg_max_iter != p0.cg_max_iter || p.reliable_every != p0.reliable_every ||
            p.reliable_delta != p0.reliable_delta) {
            set_error("chains of one context must share precision and CG settings");
            return YK_EINVAL;
        }
        if (p.pions != p0.pions) {
            set_error("chains of one context must all carry pions or none");
            return YK_EINVAL;
        }
    }
    std::unique_ptr<yk_ctx> ctx(new yk_ctx());
    YK_CK(cudaGetDevice(&ctx->dev));
    YK_CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    ctx->own_stream = true;
    YK_CK(cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking));
    YK_CK(cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming));
    YK_CK(cudaEventCreateWithFlags(&ctx->join_ev, cudaEventDisableTiming));
    YK_CK(cudaEventCreateWithFlags(&ctx->join2_ev, cudaEventDisableTiming));
    YK_CK(cudaDeviceGetAttribute(&ctx->n_sm, cudaDevAttrMultiProcessorCount, ctx->dev));
    ctx->pions = p0.pions != 0;
    ctx->precision = p0.precision;
    ctx->tol_mode = p0.cg_tol_mode;
    ctx->tol = p0.cg_tol;
    ctx->max_iter = p0.cg_max_iter;
    ctx->reliable_every = p0.reliable_every;
    ctx->reliable_delta = p0.reliable_delta;
    const bool mixed = ctx->precision == YK_MIXED;
    // occupancy queries and kernel attributes before any stream capture
    cg_max_grid(1, mixed);
    cg_max_grid(2, false);
    cg_max_grid(2, true);
    if (mixed) cg_halo_init();
    noise_init_attributes();
    {
        // opt-in while its FP64 reliable updates run on 16 SMs only
        const char* env = getenv("YK_CG_CLUSTER");
        bool want = mixed && env && env[0] == '1';
        int sites = 0;
        for (int c = 0; c < n_chains && want; ++c) {
            const yk_params& q = params[c];
            if (!cg_cluster_fits(q.Nt, q.Nx))
                want = false;
            else
                sites = std::max(sites, ((q.Nt + 15) / 16) * q.Nx);
        }
        ctx->cg_cluster = want && cg_cluster_init();
        ctx->cluster_sites = sites;
        const char* he = getenv("YK_CG_HALO");
        ctx->cg_halo = !(he && he[0] == '0');
        const char* ne = getenv("YK_NOISE_OVERLAP");
        ctx->noise_overlap = !(ne && ne[0] == '0');
        const char* ae = getenv("YK_AUTOTUNE");
        ctx->autotune = !(ae && ae[0] == '0');
        const char* be = getenv("YK_CG_BALANCE");
        ctx->cg_balance = be && be[0] == '1';
        const char* ie = getenv("YK_IO_KERNEL");
        ctx->io_kernel = !(ie && ie[0] == '0');
    }

    ctx->ch.resize(n_chains);
    int nsys = 0, nsys_tiles = 0, nsite_tiles = 0, nrows = 0, ncols = 0, nwhite = 0;
    for (int c = 0; c < n_chains; ++c) {
        Chain& C = ctx->ch[c];
        C.p = params[c];
        yk_derive_action(&C.p, &C.a);
        C.Nt = C.p.Nt;
        C.Nx = C.p.Nx;
        C.V = C.Nt * C.Nx;
        C.filter = all_modes_kept(C.Nt, C.Nx, C.p.cut_fraction) ? 0 : 1;
        // with pions the step solves complex systems (the chain's workspace)
        C.pions = C.p.pions != 0;
        C.n_rhs_pion = (C.pions && C.a.g != 0.0) ? C.p.n_rhs : 0;
        C.n_rhs_step = (!C.pions && C.a.g != 0.0) ? C.p.n_rhs : 0;
        const int nt = ntiles_of(C.V);
        C.sys0 = nsys;
        C.cg_tile0 = nsys_tiles;
        nsys += C.n_rhs_step;
        nsys_tiles += C.n_rhs_step * nt;
        C.cg_tile1 = nsys_tiles;
        C.site_tile0 = nsite_tiles;
        C.nsite_tiles = nt;
        nsite_tiles += nt;
        if (C.filter) {
            C.row0 = nrows;
            C.nrows = (C.Nt + 1) / 2;   // row pairs
            nrows += C.nrows;
            const int cw = noise_strip(C.Nt);
            C.col0 = ncols;
            C.ncols = (int)kept_strips(C.Nt, C.Nx, C.p.cut_fraction, cw).size();
            ncols += C.ncols;
            if (C.Nx > ctx->max_nx) ctx->max_nx = C.Nx;
            const int ce = C.Nt * (cw < C.Nx ? cw : C.Nx);
            if (ce > ctx->max_cols) ctx->max_cols = ce;
        } else {
            C.white0 = nwhite;
            C.nwhite = nt;
            nwhite += nt;
        }
    }
    ctx->nsys = nsys;
    ctx->n_sys_tiles = nsys_tiles;
    ctx->n_site_tiles = nsite_tiles;
    ctx->nrows = nrows;
    ctx->ncols = ncols;
    ctx->nwhite = nwhite;

    // ---- one arena for everything
    Arena ar;
    struct COff {
        size_t phi, drift, xi, force, slices, spec, keep, twt, twx;
    };
    std::vector<COff> co(n_chains);
    struct SOff {
        size_t b, x, r0, r1, p0, p1, t64, ap64, s0, s1, q0, q1, t32, ap32, xs, diag, eta0, eta1, tag;
    };
    std::vector<SOff> so(nsys);
    for (int c = 0; c < n_chains; ++c) {
        Chain& C = ctx->ch[c];
        const size_t V = C.V;
        co[c].phi = ar.reserve(8 * V);
        co[c].drift = ar.reserve(8 * V);
        co[c].xi = ar.reserve(8 * V);
        co[c].force = ar.reserve(8 * V);
        co[c].slices = ar.reserve(8 * (size_t)C.Nt);
        if (C.filter) {
            co[c].spec = ar.reserve(16 * V);
            co[c].keep = ar.reserve(V);
            co[c].twt = ar.reserve(16 * (size_t)C.Nt);
            co[c].twx = ar.reserve(16 * (size_t)C.Nx);
        }
        for (int j = 0; j < C.n_rhs_step; ++j) {
            SOff& o = so[C.sys0 + j];
            const size_t d = 8 * 4 * V, f = 4 * 4 * V;
            o.b = ar.reserve(d);
            o.x = ar.reserve(d);
            o.t64 = ar.reserve(d);
            o.eta0 = ar.reserve(d);
            o.eta1 = ar.reserve(d);
            o.tag = ar.reserve(2 * sizeof(int64_t));
            if (mixed) {
                o.s0 = ar.reserve(f);
                o.s1 = ar.reserve(f);
                o.q0 = ar.reserve(f);
                o.q1 = ar.reserve(f);
                o.t32 = ar.reserve(f);
                o.ap32 = ar.reserve(f);
                o.xs = ar.reserve(f);
                o.diag = ar.reserve(sizeof(float) * V);
            } else {
                o.r0 = ar.reserve(d);
                o.r1 = ar.reserve(d);
                o.p0 = ar.reserve(d);
                o.p1 = ar.reserve(d);
                o.ap64 = ar.reserve(d);
            }
        }
    }
    const size_t o_chains = ar.reserve(sizeof(ChainDev) * n_chains);
    const size_t o_sys = ar.reserve(sizeof(SysDev) * (nsys > 0 ? nsys : 1));
    const size_t o_systiles = ar.reserve(sizeof(int2) * (nsys_tiles > 0 ? nsys_tiles : 1));
    const size_t o_state = ar.reserve(sizeof(CGState) * (nsys > 0 ? nsys : 1));
    const size_t o_partial = ar.reserve(sizeof(Partial) * (nsys_tiles > 0 ? nsys_tiles : 1));
    const size_t o_coef = ar.reserve(sizeof(CGCoef) * (nsys > 0 ? nsys : 1));
    const size_t o_flags = ar.reserve(sizeof(unsigned) * kFlagStride * (size_t)kMaxGrid);
    const size_t o_bar = ar.reserve(sizeof(GridBarrier));
    const size_t o_err = ar.reserve(sizeof(int) * 4);
    const size_t o_balance = ar.reserve(sizeof(int) * (kMaxGrid + 2));
    const size_t o_sitetiles = ar.reserve(sizeof(int2) * nsite_tiles);
    const size_t o_tmax = ar.reserve(sizeof(double) * nsite_tiles);
    const size_t o_tsum = ar.reserve(sizeof(double2) * nsite_tiles);
    const size_t o_tsum2 = ar.reserve(sizeof(double) * nsite_tiles);
    const size_t o_rows = ar.reserve(sizeof(int2) * (nrows > 0 ? nrows : 1));
    const size_t o_cols = ar.reserve(sizeof(int2) * (ncols > 0 ? ncols : 1));
    const size_t o_white = ar.reserve(sizeof(int2) * (nwhite > 0 ? nwhite : 1));
    if (cudaMalloc(&ctx->mem, ar.used) != cudaSuccess) {
        cudaGetLastError();
        set_error("context allocation of %zu bytes failed", ar.used);
        cudaStreamDestroy(ctx->stream);
        cudaStreamDestroy(ctx->aux);
        cudaEventDestroy(ctx->fork_ev);
        cudaEventDestroy(ctx->join_ev);
        cudaEventDestroy(ctx->join2_ev);
        return YK_ENOMEM;
    }
    ar.base = (char*)ctx->mem;
    YK_CK(cudaMemsetAsync(ctx->mem, 0, ar.used, ctx->stream));
    // the synchronous uploads below run on the legacy stream, which does not
    // wait for the context's non-blocking stream
    YK_CK(cudaStreamSynchronize(ctx->stream));

    ctx->d_chains = ar.at<ChainDev>(o_chains);
    ctx->d_sys = ar.at<SysDev>(o_sys);
    ctx->d_sys_tiles = ar.at<int2>(o_systiles);
    ctx->d_state = ar.at<CGState>(o_state);
    ctx->d_partial = ar.at<Partial>(o_partial);
    ctx->d_coef = ar.at<CGCoef>(o_coef);
    ctx->d_flags = ar.at<unsigned>(o_flags);
    ctx->d_bar = ar.at<GridBarrier>(o_bar);
    ctx->d_err = ar.at<int>(o_err);
    ctx->d_nactive = ctx->d_err + 1;
    ctx->d_anyru = ctx->d_err + 2;
    ctx->d_balance = ar.at<int>(o_balance);
    ctx->d_site_tiles = ar.at<int2>(o_sitetiles);
    ctx->d_tile_max = ar.at<double>(o_tmax);
    ctx->d_tile_sum = ar.at<double2>(o_tsum);
    ctx->d_tile_sum2 = ar.at<double>(o_tsum2);
    ctx->d_rows = ar.at<int2>(o_rows);
    ctx->d_cols = ar.at<int2>(o_cols);
    ctx->d_white = ar.at<int2>(o_white);

    std::vector<SysDev> hs(nsys);
    std::vector<int2> sys_tiles, site_tiles, rows, cols, white;
    ctx->h_chains.assign(n_chains, ChainDev());
    int64_t drand_skip = 0;
    for (int c = 0; c < n_chains; ++c) {
        Chain& C = ctx->ch[c];
        const COff& o = co[c];
        C.phi = ar.at<double>(o.phi);
        C.drift = ar.at<double>(o.drift);
        C.xi = ar.at<double>(o.xi);
        C.force = ar.at<double>(o.force);
        C.slices = ar.at<double>(o.slices);
        C.spec = C.filter ? ar.at<double2>(o.spec) : nullptr;
        C.keep = C.filter ? ar.at<uint8_t>(o.keep) : nullptr;
        C.tw_t = C.filter ? ar.at<double2>(o.twt) : nullptr;
        C.tw_x = C.filter ? ar.at<double2>(o.twx) : nullptr;
        const int nt = ntiles_of(C.V);
        for (int t = 0; t < nt; ++t) site_tiles.push_back(make_int2(c, t * kTile));
        for (int j = 0; j < C.n_rhs_step; ++j) {
            const SOff& q = so[C.sys0 + j];
            SysDev& S = hs[C.sys0 + j];
            std::memset(&S, 0, sizeof(S));
            S.chain = c;
            S.rhs = j;
            S.Nt = C.Nt;
            S.Nx = C.Nx;
            S.V = C.V;
            S.tile0 = (int)sys_tiles.size();
            S.ntiles = nt;
            S.m0 = C.a.m0;
            S.g = C.a.g;
            S.r = C.a.r;
            S.sigma = C.phi;
            S.b = ar.at<double>(q.b);
            S.x = ar.at<double>(q.x);
            S.t64 = ar.at<double>(q.t64);
            if (mixed) {
                S.r32[0] = ar.at<float>(q.s0);
                S.r32[1] = ar.at<float>(q.s1);
                S.p32[0] = ar.at<float>(q.q0);
                S.p32[1] = ar.at<float>(q.q1);
                S.t32 = ar.at<float>(q.t32);
                S.Ap32 = ar.at<float>(q.ap32);
                S.xs32 = ar.at<float>(q.xs);
                S.diag32 = ar.at<float>(q.diag);
            } else {
                S.r64[0] = ar.at<double>(q.r0);
                S.r64[1] = ar.at<double>(q.r1);
                S.p64[0] = ar.at<double>(q.p0);
                S.p64[1] = ar.at<double>(q.p1);
                S.Ap64 = ar.at<double>(q.ap64);
            }
            S.gen_eta = 1;
            S.seed = (uint64_t)C.p.seed;
            S.step = &ctx->d_chains[c].step;
            S.eta_ahead[0] = ar.at<double>(q.eta0);
            S.eta_ahead[1] = ar.at<double>(q.eta1);
            S.eta_tag = ar.at<int64_t>(q.tag);
            YK_CK(cudaMemsetAsync(S.eta_tag, 0xff, 2 * sizeof(int64_t), ctx->stream));   // -1: holds no step
            for (int t = 0; t < nt; ++t) sys_tiles.push_back(make_int2(C.sys0 + j, t * kTile));
        }
        if (C.filter) {
            for (int t = 0; t < C.Nt; t += 2) rows.push_back(make_int2(c, t));
            for (int x0 : kept_strips(C.Nt, C.Nx, C.p.cut_fraction, noise_strip(C.Nt))) cols.push_back(make_int2(c, x0));
            std::vector<uint8_t> keep;
            momentum_keep(C.Nt, C.Nx, C.p.cut_fraction, keep);
            std::vector<double> twt, twx;
            twiddles(C.Nt, twt);
            twiddles(C.Nx, twx);
            YK_CK(cudaMemcpy(C.keep, keep.data(), keep.size(), cudaMemcpyHostToDevice));
            YK_CK(cudaMemcpy(C.tw_t, twt.data(), sizeof(double) * twt.size(), cudaMemcpyHostToDevice));
            YK_CK(cudaMemcpy(C.tw_x, twx.data(), sizeof(double) * twx.size(), cudaMemcpyHostToDevice));
        } else {
            for (int t = 0; t < nt; ++t) white.push_back(make_int2(c, t * kTile));
        }
        // initial field (main.cu:92-95)
        std::vector<double> phi(C.V, 0.0);
        if (C.p.init == YK_INIT_DRAND48) {
            drand48_field(drand_skip, C.V, phi.data());
            drand_skip += C.V;
        } else if (C.p.init == YK_INIT_PHILOX) {
            // 1 - 2u, u uniform in (0, 1) from Philox stream kind 0 of (seed, chain)
            philox_uniform_field((uint64_t)C.p.seed, (uint32_t)c, C.V, phi.data());
        }
        YK_CK(cudaMemcpy(C.phi, phi.data(), sizeof(double) * C.V, cudaMemcpyHostToDevice));

        ChainDev& H = ctx->h_chains[c];
        std::memset(&H, 0, sizeof(H));
        H.Nt = C.Nt;
        H.Nx = C.Nx;
        H.V = C.V;
        H.n_rhs = C.n_rhs_step;
        H.sys0 = C.sys0;
        H.tile0 = C.site_tile0;
        H.ntiles = C.nsite_tiles;
        H.m2 = C.a.m2;
        H.lambda = C.a.lambda;
        H.lambda6 = C.a.lambda / 6.0;
        H.g = C.a.g;
        H.m0 = C.a.m0;
        H.r = C.a.r;
        H.cut = C.a.cut_fraction;
        H.eps_bar = C.a.eps_bar;
        H.fixed_dt = C.p.fixed_dt;
        H.drift_mode = C.a.drift_mode;
        H.filter = C.filter;
        H.seed = (uint64_t)C.p.seed;
        H.chain_id = (uint32_t)c;
        H.phi = C.phi;
        H.drift = C.drift;
        H.xi = C.xi;
        H.white = nullptr;
        H.spec = C.spec;
        H.keep = C.keep;
        H.tw_t = C.tw_t;
        H.tw_x = C.tw_x;
        H.step = 0;
        H.time = 0.0;
    }
    YK_CK(cudaMemcpyAsync(ctx->d_chains, ctx->h_chains.data(), sizeof(ChainDev) * n_chains,
                          cudaMemcpyHostToDevice, ctx->stream));
    if (nsys > 0) {
        YK_CK(cudaMemcpyAsync(ctx->d_sys, hs.data(), sizeof(SysDev) * nsys, cudaMemcpyHostToDevice, ctx->stream));
        YK_CK(cudaMemcpyAsync(ctx->d_sys_tiles, sys_tiles.data(), sizeof(int2) * sys_tiles.size(),
                              cudaMemcpyHostToDevice, ctx->stream));
    }
    YK_CK(cudaMemcpyAsync(ctx->d_site_tiles, site_tiles.data(), sizeof(int2) * site_tiles.size(),
                          cudaMemcpyHostToDevice, ctx->stream));
    if (!rows.empty()) {
        YK_CK(cudaMemcpyAsync(ctx->d_rows, rows.data(), sizeof(int2) * rows.size(), cudaMemcpyHostToDevice,
                              ctx->stream));
        YK_CK(cudaMemcpyAsync(ctx->d_cols, cols.data(), sizeof(int2) * cols.size(), cudaMemcpyHostToDevice,
                              ctx->stream));
    }
    if (!white.empty())
        YK_CK(cudaMemcpyAsync(ctx->d_white, white.data(), sizeof(int2) * white.size(), cudaMemcpyHostToDevice,
                              ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->pions)
        if (int rc = pion_setup(ctx.get())) {
            yk_ctx_destroy(ctx.release());
            return rc;
        }
    if (int rc = eo_setup(ctx.get(), hs)) {
        yk_ctx_destroy(ctx.release());
        return rc;
    }
    *out = ctx.release();
    return YK_OK;
}

int yk_ctx_destroy(yk_ctx* ctx)
{
    if (!ctx) return YK_OK;
    cudaStreamSynchronize(ctx->stream);
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    for (auto& g : ctx->io) cudaGraphExecDestroy(g.exec);
    if (ctx->io_pin) cudaFreeHost(ctx->io_pin);
    for (auto& r : ctx->recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (auto e : ctx->pool) cudaEventDestroy(e);
    for (auto& C : ctx->ch) {
        if (C.ws.mem) cudaFree(C.ws.mem);
        if (C.series) cudaFree(C.series);
        net_destroy(C.net);
        net_destroy(C.pcg_ws);
    }
    if (ctx->mem) cudaFree(ctx->mem);
    if (ctx->pion_mem) cudaFree(ctx->pion_mem);
    if (ctx->eo_mem) cudaFree(ctx->eo_mem);
    if (ctx->aux) {
        cudaStreamSynchronize(ctx->aux);
        cudaStreamDestroy(ctx->aux);
    }
    if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
    if (ctx->join_ev) cudaEventDestroy(ctx->join_ev);
    if (ctx->join2_ev) cudaEventDestroy(ctx->join2_ev);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return YK_OK;
}

int yk_ctx_set_stream(yk_ctx* ctx, void* stream)
{
    if (!ctx) return YK_EINVAL;
    YK_CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    ctx->own_stream = false;
    ctx->stream = (cudaStream_t)stream;
    return YK_OK;
}

int yk_check_wait_timeout(void* stream, int* status)
{
    int st = 0;
    if (wait_timeout_probe(static_cast<cudaStream_t>(stream), &st) != 0) {
        set_error("yk_check_wait_timeout: %s", cudaGetErrorString(cudaGetLastError()));
        return YK_ECUDA;
    }
    if (status) *status = st;
    if (st == YK_ETIMEOUT) {
        set_error("the probe's bounded wait gave up (as designed)");
        return YK_ETIMEOUT;
    }
    return YK_OK;
}

int yk_ctx_synchronize(yk_ctx* ctx)
{
    if (!ctx) return YK_EINVAL;
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return status_of_err(ctx);
}

int yk_ctx_n_chains(const yk_ctx* ctx) { return ctx ? (int)ctx->ch.size() : 0; }

int yk_ctx_volume(const yk_ctx* ctx, int chain)
{
    if (!ctx || chain < 0 || chain >= (int)ctx->ch.size()) return 0;
    return ctx->ch[chain].V;
}

int yk_ctx_shape(const yk_ctx* ctx, int c, int* Nt, int* Nx)
{
    if (!ctx || c < 0 || c >= (int)ctx->ch.size()) return YK_EINVAL;
    if (Nt) *Nt = ctx->ch[c].Nt;
    if (Nx) *Nx = ctx->ch[c].Nx;
    return YK_OK;
}

int yk_set_field_host(yk_ctx* ctx, int c, const double* phi)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    YK_CK(cudaMemcpyAsync(ctx->ch[c].phi, phi, sizeof(double) * ctx->ch[c].V, cudaMemcpyHostToDevice, ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return YK_OK;
}

int yk_get_field_host(yk_ctx* ctx, int c, double* phi)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    YK_CK(cudaMemcpyAsync(phi, ctx->ch[c].phi, sizeof(double) * ctx->ch[c].V, cudaMemcpyDeviceToHost, ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return YK_OK;
}

int yk_series_record(yk_ctx* ctx, int c, int64_t capacity)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    if (capacity < 0) {
        set_error("yk_series_record: negative capacity");
        return YK_EINVAL;
    }
    Chain& C = ctx->ch[c];
    YK_CK(cudaStreamSynchronize(ctx->stream));
    if (C.series) {
        YK_CK(cudaFree(C.series));
        C.series = nullptr;
        C.series_cap = 0;
    }
    if (capacity > 0) {
        if (cudaMalloc(&C.series, sizeof(double) * (size_t)capacity) != cudaSuccess) {
            cudaGetLastError();
            C.series = nullptr;
            set_error("yk_series_record: allocation of %lld values failed", (long long)capacity);
            return YK_ENOMEM;
        }
        C.series_cap = capacity;
    }
    // the update kernels read these three fields of the device record
    ChainDev& H = ctx->h_chains[c];
    H.series = C.series;
    H.series_cap = C.series_cap;
    H.series_n = 0;
    const size_t off = offsetof(ChainDev, series);
    const size_t len = offsetof(ChainDev, series_n) + sizeof(int64_t) - off;
    YK_CK(cudaMemcpyAsync(reinterpret_cast<char*>(ctx->d_chains + c) + off, reinterpret_cast<const char*>(&H) + off,
                          len, cudaMemcpyHostToDevice, ctx->stream));
    if (ctx->pions)
        for (int a = 0; a < 3; ++a)
            YK_CK(cudaMemcpyAsync(reinterpret_cast<char*>(ctx->d_pchains + (size_t)a * ctx->ch.size() + c) + off,
                                  reinterpret_cast<const char*>(&H) + off, len, cudaMemcpyHostToDevice,
                                  ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return YK_OK;
}

int yk_series_read(yk_ctx* ctx, int c, double* host, int64_t cap, int64_t* n)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    if (!n || (cap > 0 && !host)) {
        set_error("yk_series_read: bad arguments");
        return YK_EINVAL;
    }
    const Chain& C = ctx->ch[c];
    int64_t have = 0;
    if (C.series)
        YK_CK(cudaMemcpyAsync(&have, &ctx->d_chains[c].series_n, sizeof(int64_t), cudaMemcpyDeviceToHost,
                              ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    if (!host) {   // a query of how many values are recorded
        *n = have;
        return YK_OK;
    }
    const int64_t k = std::min(have, cap);
    if (k > 0) {
        YK_CK(cudaMemcpyAsync(host, C.series, sizeof(double) * (size_t)k, cudaMemcpyDeviceToHost, ctx->stream));
        YK_CK(cudaStreamSynchronize(ctx->stream));
    }
    *n = k;
    return YK_OK;
}

int yk_series_analyse(yk_ctx* ctx, int c, double stau, yk_series_stats* out)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    const Chain& C = ctx->ch[c];
    if (!out || !(stau > 0.0) || !C.series) {
        set_error("yk_series_analyse: %s", C.series ? "bad arguments" : "no series is recorded (yk_series_record)");
        return YK_EINVAL;
    }
    int64_t have = 0;
    YK_CK(cudaMemcpyAsync(&have, &ctx->d_chains[c].series_n, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return series_analyse(C.series, have, C.V, stau, out, ctx->stream);
}

int yk_set_pions_host(yk_ctx* ctx, int c, const double* pi)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    const Chain& C = ctx->ch[c];
    if (!C.pions || !pi) {
        set_error("yk_set_pions_host: %s", C.pions ? "null buffer" : "the context carries no pions");
        return YK_EINVAL;
    }
    YK_CK(cudaMemcpyAsync(C.pi, pi, sizeof(double) * 3 * (size_t)C.V, cudaMemcpyHostToDevice, ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return YK_OK;
}

int yk_get_pions_host(yk_ctx* ctx, int c, double* pi)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    const Chain& C = ctx->ch[c];
    if (!C.pions || !pi) {
        set_error("yk_get_pions_host: %s", C.pions ? "null buffer" : "the context carries no pions");
        return YK_EINVAL;
    }
    YK_CK(cudaMemcpyAsync(pi, C.pi, sizeof(double) * 3 * (size_t)C.V, cudaMemcpyDeviceToHost, ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return YK_OK;
}

int yk_pions_device(yk_ctx* ctx, int c, double** pi)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    if (!ctx->ch[c].pions || !pi) {
        set_error("yk_pions_device: the context carries no pions");
        return YK_EINVAL;
    }
    *pi = ctx->ch[c].pi;
    return YK_OK;
}

int yk_field_device(yk_ctx* ctx, int c, double** phi)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    *phi = ctx->ch[c].phi;
    return YK_OK;
}

int yk_dirac_apply(yk_ctx* ctx, int c, const void* in, void* out, int dagger, int precision)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    if (!in || !out || (precision != YK_FP64 && precision != YK_FP32)) {
        set_error("yk_dirac_apply: bad buffers or precision");
        return YK_EINVAL;
    }
    if (in == out) {
        set_error("yk_dirac_apply: in and out must not alias");
        return YK_EINVAL;
    }
    const Chain& C = ctx->ch[c];
    YK_CK(launch_dirac(in, out, C.phi, C.Nt, C.Nx, C.a.m0, C.a.g, C.a.r, dagger ? 1 : 0, precision, 2,
                       ctx->stream, C.pions ? C.pi : nullptr));
    return YK_OK;
}

int yk_cg_solve(yk_ctx* ctx, int c, const void* b, void* x, int mtype, double tol, int tol_mode, int max_iter,
                int precision, yk_solve_stats* stats)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    if (!b || !x || b == x || (precision != YK_FP64 && precision != YK_MIXED) || max_iter < 0 ||
        (mtype != YK_NORMAL && mtype != YK_DAGGER) || !(tol >= 0.0)) {
        set_error("yk_cg_solve: bad arguments");
        return YK_EINVAL;
    }
    if (int rc = ensure_ws(ctx, c, 1)) return rc;
    Workspace& w = ctx->ch[c].ws;
    w.h_sys[0].b = (double*)b;
    w.h_sys[0].x = (double*)x;
    int rc = ws_solve(ctx, c, 1, mtype, tol, tol_mode, max_iter, precision, stats);
    w.h_sys[0].b = nullptr;
    return rc;
}

int yk_fermion_force(yk_ctx* ctx, int c, const void* eta, double* F, yk_solve_stats* stats)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    if (!F) {
        set_error("yk_fermion_force: F is null");
        return YK_EINVAL;
    }
    Chain& C = ctx->ch[c];
    if (C.pions) {
        // F: 4V doubles (sigma, pi_1, pi_2, pi_3)
        int rc = pion_solve(ctx, c, 2, static_cast<const double*>(eta), eta ? YK_FP64 : ctx->precision, stats);
        if (rc && rc != YK_ENOCONV) return rc;
        YK_CK(launch_pion_force(ctx->d_chains + c, C.ws.d_sys, C.n_rhs_pion, C.pi, F, C.V, ctx->stream));
        YK_CK(cudaStreamSynchronize(ctx->stream));
        return rc;
    }
    if (eta) {
        const int R = C.p.n_rhs;
        if (int rc = ensure_ws(ctx, c, R)) return rc;
        Workspace& w = C.ws;
        for (int j = 0; j < R; ++j) w.h_sys[j].b = (double*)eta + (size_t)j * 8 * C.V;
        int rc = YK_OK;
        if (C.a.g != 0.0) rc = ws_solve(ctx, c, R, YK_DAGGER, ctx->tol, ctx->tol_mode, ctx->max_iter, YK_FP64, stats);
        else if (stats) *stats = yk_solve_stats{0, 0, 0.0, 0.0, 1};
        if (rc && rc != YK_ENOCONV) return rc;
        ChainDev H = ctx->h_chains[c];
        H.sys0 = 0;
        H.n_rhs = (C.a.g != 0.0) ? R : 0;
        H.drift = F;
        H.tile0 = 0;
        YK_CK(cudaMemcpyAsync(w.d_chain, &H, sizeof(ChainDev), cudaMemcpyHostToDevice, ctx->stream));
        StepArgs s = step_args(ctx);
        s.ch = w.d_chain;
        s.nch = 1;
        s.tiles = w.d_site_tiles;
        s.ntiles = ntiles_of(C.V);
        YK_CK(launch_force_drift(s, w.d_sys, 1, 2, ctx->stream));
        YK_CK(cudaStreamSynchronize(ctx->stream));
        return rc;
    }
    int rc = chain_solve(ctx, c, 2, stats);
    if (rc && rc != YK_ENOCONV) return rc;
    StepArgs s = chain_step_args(ctx, c);
    // the solve's states: chi from t64 where the solve left it there
    YK_CK(launch_force_drift(s, ctx->d_sys, 1, 1, ctx->stream, ctx->d_state));
    YK_CK(cudaMemcpyAsync(F, C.drift, sizeof(double) * C.V, cudaMemcpyDeviceToDevice, ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return rc;
}

int yk_coloured_noise(yk_ctx* ctx, int c, const double* white, double* xi)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    if (!xi) {
        set_error("yk_coloured_noise: xi is null");
        return YK_EINVAL;
    }
    Chain& C = ctx->ch[c];
    NoiseTables nt = {ctx->d_rows + C.row0, C.nrows, ctx->d_cols + C.col0, C.ncols, ctx->d_white + C.white0,
                      C.nwhite};
    YK_CK(launch_noise_tables(ctx->d_chains, nt, ctx->max_nx, ctx->max_cols, white, ctx->stream));
    YK_CK(cudaMemcpyAsync(xi, C.xi, sizeof(double) * C.V, cudaMemcpyDeviceToDevice, ctx->stream));
    return YK_OK;
}

int yk_langevin_step(yk_ctx* ctx, int n_steps)
{
    if (!ctx || n_steps < 0) {
        set_error("yk_langevin_step: bad arguments");
        return YK_EINVAL;
    }
    if (ctx->pions) {
        for (int i = 0; i < n_steps; ++i)
            for (int c = 0; c < (int)ctx->ch.size(); ++c)
                if (int rc = pion_step(ctx, c)) return rc;
        return YK_OK;
    }
    if (!ctx->gexec && ctx->autotune && !ctx->tuned && n_steps > 0)
        if (int rc = run_autotune(ctx)) return rc;
    if (!ctx->gexec && !ctx->graph_failed && ctx->stream) {
        cudaGraph_t g = nullptr;
        bool ok = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            // the graph holds no profiling events (profiled steps run uncaptured)
            const bool profiling = ctx->profiling;
            ctx->profiling = false;
            const int rc = enqueue_step(ctx);
            ctx->profiling = profiling;
            const bool end_ok = cudaStreamEndCapture(ctx->stream, &g) == cudaSuccess;
            ok = (rc == YK_OK) && end_ok && g;
            if (ok) ok = cudaGraphInstantiate(&ctx->gexec, g, 0) == cudaSuccess;
            if (g) cudaGraphDestroy(g);
        }
        if (!ok) {
            cudaGetLastError();
            ctx->gexec = nullptr;
            ctx->graph_failed = true;
        }
    }
    for (int i = 0; i < n_steps; ++i) {
        if (ctx->gexec && !ctx->profiling) {
            YK_CK(cudaGraphLaunch(ctx->gexec, ctx->stream));
        } else {
            if (int rc = enqueue_step(ctx)) return rc;
        }
    }
    return YK_OK;
}

namespace {

// Pinned host memory (nullptr: no copy), with its device address when it is
// mapped (else *dev = nullptr).
bool pinned_host(const void* p, void** dev)
{
    *dev = nullptr;
    if (!p) return true;
    cudaPointerAttributes at = {};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (at.type != cudaMemoryTypeHost) return false;
    *dev = at.devicePointer;
    return true;
}

static_assert(sizeof(yk_obs) % 8 == 0, "the observables are copied as 8-byte words");

// The io graph of (c, in, out): found, or captured (the least recently used
// of four replaced); nullptr when capture fails (the calls are then issued
// one by one).
yk_ctx::IoGraph* io_graph(yk_ctx* ctx, int c, const double* in, double* out, void* in_dev, void* out_dev)
{
    ++ctx->io_clock;
    for (auto& g : ctx->io)
        if (g.c == c && g.in == in && g.out == out && g.in_dev == in_dev && g.out_dev == out_dev) {
            g.used = ctx->io_clock;
            return &g;
        }
    if (ctx->io_failed) return nullptr;
    if (!ctx->io_pin && cudaMallocHost(&ctx->io_pin, sizeof(yk_obs) + sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        ctx->io_pin = nullptr;
        ctx->io_failed = true;
        return nullptr;
    }
    const Chain& C = ctx->ch[c];
    yk_obs* hobs = static_cast<yk_obs*>(ctx->io_pin);
    int* herr = reinterpret_cast<int*>(hobs + 1);
    void* pin_dev = nullptr;
    if (cudaHostGetDevicePointer(&pin_dev, ctx->io_pin, 0) != cudaSuccess) {
        cudaGetLastError();
        pin_dev = nullptr;
    }
    // kernels through the mapped buffers, else copy-engine copies
    const bool kern = ctx->io_kernel && pin_dev && (!in || in_dev) && (!out || out_dev);
    cudaGraph_t g = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool ok = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
        bool rec = true;
        if (in)
            rec = (kern ? launch_io_load(static_cast<const double*>(in_dev), C.phi, C.V, ctx->stream)
                        : cudaMemcpyAsync(C.phi, in, sizeof(double) * C.V, cudaMemcpyHostToDevice, ctx->stream)) ==
                  cudaSuccess;
        if (rec) rec = enqueue_step(ctx) == YK_OK;
        if (rec && kern) {
            yk_obs* dobs = static_cast<yk_obs*>(pin_dev);
            rec = launch_io_store(C.phi, static_cast<double*>(out_dev), C.V, &ctx->d_chains[c].obs, dobs,
                                  sizeof(yk_obs), ctx->d_err, reinterpret_cast<int*>(dobs + 1), ctx->stream) ==
                  cudaSuccess;
        } else if (rec) {
            if (out)
                rec = cudaMemcpyAsync(out, C.phi, sizeof(double) * C.V, cudaMemcpyDeviceToHost, ctx->stream) ==
                      cudaSuccess;
            if (rec)
                rec = cudaMemcpyAsync(hobs, &ctx->d_chains[c].obs, sizeof(yk_obs), cudaMemcpyDeviceToHost,
                                      ctx->stream) == cudaSuccess;
            if (rec)
                rec = cudaMemcpyAsync(herr, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream) ==
                      cudaSuccess;
        }
        const bool end_ok = cudaStreamEndCapture(ctx->stream, &g) == cudaSuccess;
        ok = rec && end_ok && g && cudaGraphInstantiate(&exec, g, 0) == cudaSuccess;
        if (g) cudaGraphDestroy(g);
    }
    if (!ok) {
        cudaGetLastError();
        if (exec) cudaGraphExecDestroy(exec);
        ctx->io_failed = true;
        return nullptr;
    }
    if (ctx->io.size() >= 4) {
        auto lru = std::min_element(ctx->io.begin(), ctx->io.end(),
                                    [](const yk_ctx::IoGraph& a, const yk_ctx::IoGraph& b) { return a.used < b.used; });
        cudaGraphExecDestroy(lru->exec);
        ctx->io.erase(lru);
    }
    ctx->io.push_back({c, in, out, in_dev, out_dev, exec, ctx->io_clock});
    return &ctx->io.back();
}

}  // namespace

int yk_langevin_step_io(yk_ctx* ctx, int c, const double* phi_in, double* phi_out, yk_obs* obs)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    const Chain& C = ctx->ch[c];
    // after the first step (autotuning, the step graph): one graph launch and
    // one synchronisation when the host fields are pinned
    void *in_dev = nullptr, *out_dev = nullptr;
    if (ctx->gexec && !ctx->pions && !ctx->profiling && pinned_host(phi_in, &in_dev) && pinned_host(phi_out, &out_dev)) {
        if (yk_ctx::IoGraph* g = io_graph(ctx, c, phi_in, phi_out, in_dev, out_dev)) {
            YK_CK(cudaGraphLaunch(g->exec, ctx->stream));
            YK_CK(cudaStreamSynchronize(ctx->stream));
            const yk_obs* hobs = static_cast<const yk_obs*>(ctx->io_pin);
            if (obs) *obs = *hobs;
            if (const int e = *reinterpret_cast<const int*>(hobs + 1)) {
                set_error("a bounded device wait gave up (status %d)", e);
                return YK_ETIMEOUT;
            }
            return YK_OK;
        }
    }
    if (phi_in)
        YK_CK(cudaMemcpyAsync(C.phi, phi_in, sizeof(double) * C.V, cudaMemcpyHostToDevice, ctx->stream));
    if (int rc = yk_langevin_step(ctx, 1)) return rc;
    if (phi_out)
        YK_CK(cudaMemcpyAsync(phi_out, C.phi, sizeof(double) * C.V, cudaMemcpyDeviceToHost, ctx->stream));
    if (obs) YK_CK(cudaMemcpyAsync(obs, &ctx->d_chains[c].obs, sizeof(yk_obs), cudaMemcpyDeviceToHost, ctx->stream));
    return status_of_err(ctx);   // the one synchronisation
}

int yk_euler_update(yk_ctx* ctx, int c, const double* force, const double* xi, yk_obs* obs)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    if (int rc = no_pions(ctx, "yk_euler_update")) return rc;
    if (!force || !xi) {
        set_error("yk_euler_update: force and xi are required");
        return YK_EINVAL;
    }
    Chain& C = ctx->ch[c];
    YK_CK(cudaMemcpyAsync(C.drift, force, sizeof(double) * C.V, cudaMemcpyDeviceToDevice, ctx->stream));
    YK_CK(cudaMemcpyAsync(C.xi, xi, sizeof(double) * C.V, cudaMemcpyDeviceToDevice, ctx->stream));
    StepArgs s = chain_step_args(ctx, c);
    YK_CK(launch_force_drift(s, ctx->d_sys, 2, 1, ctx->stream));
    YK_CK(launch_update(s, ctx->d_state, ctx->stream));
    if (obs) return yk_observables(ctx, c, obs);
    return YK_OK;
}

int yk_profile_begin(yk_ctx* ctx)
{
    if (int rc = no_pions(ctx, "yk_profile_begin")) return rc;
    if (!ctx) return YK_EINVAL;
    YK_CK(cudaStreamSynchronize(ctx->stream));
    ctx->profiling = true;
    ctx->recs.clear();
    ctx->prof_steps = 0;
    ctx->prof_launches = 0;
    ctx->prof_iters0.assign(ctx->ch.size(), 0);
    for (size_t c = 0; c < ctx->ch.size(); ++c) {
        yk_obs o;
        if (int rc = yk_observables(ctx, (int)c, &o)) return rc;
        ctx->prof_iters0[c] = o.cg_iterations_total;
    }
    return YK_OK;
}

int yk_profile_end(yk_ctx* ctx, yk_profile* out)
{
    if (!ctx || !out) return YK_EINVAL;
    YK_CK(cudaStreamSynchronize(ctx->stream));
    std::memset(out, 0, sizeof(*out));
    for (auto& r : ctx->recs) {
        float ms = 0.f;
        YK_CK(cudaEventElapsedTime(&ms, r.a, r.b));
        if (r.cls == 0) out->noise_ms += ms;
        if (r.cls == 1) {
            out->cg_ms += ms;
            out->cg_launches += 1;
        }
        if (r.cls == 2) out->force_ms += ms;
        if (r.cls == 3) out->update_ms += ms;
        ctx->pool.push_back(r.a);
        ctx->pool.push_back(r.b);
    }
    ctx->recs.clear();
    out->steps = ctx->prof_steps;
    out->launches = ctx->prof_launches;
    for (size_t c = 0; c < ctx->ch.size(); ++c) {
        yk_obs o;
        if (int rc = yk_observables(ctx, (int)c, &o)) return rc;
        const int64_t it = o.cg_iterations_total - ctx->prof_iters0[c];
        out->cg_iterations += it;
        out->cg_site_iterations += it * (int64_t)ctx->ch[c].V;
        out->sites += (int64_t)ctx->ch[c].V;
    }
    out->cg_grid = ctx->cg_grid;
    out->cg_kernel = ctx->cg_kernel;
    ctx->profiling = false;
    return YK_OK;
}

int yk_observables(yk_ctx* ctx, int c, yk_obs* obs)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    YK_CK(cudaMemcpyAsync(obs, &ctx->d_chains[c].obs, sizeof(yk_obs), cudaMemcpyDeviceToHost, ctx->stream));
    return status_of_err(ctx);
}

int yk_time_slices(yk_ctx* ctx, int c, double* slices)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    Chain& C = ctx->ch[c];
    YK_CK(launch_time_slices(C.phi, C.slices, C.Nt, C.Nx, ctx->stream));
    YK_CK(cudaMemcpyAsync(slices, C.slices, sizeof(double) * C.Nt, cudaMemcpyDeviceToHost, ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return YK_OK;
}

int yk_correlator(yk_ctx* ctx, int c, double* corr, yk_solve_stats* stats)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    if (int rc = ensure_ws(ctx, c, 1)) return rc;
    Chain& C = ctx->ch[c];
    Workspace& w = C.ws;
    // point source in[0] = in[1] = 1 at site 0 (main.cu:441-450)
    YK_CK(cudaMemsetAsync(w.point, 0, sizeof(double) * 8 * (size_t)C.V, ctx->stream));
    const double one = 1.0;
    YK_CK(cudaMemcpyAsync(w.point + 0, &one, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    YK_CK(cudaMemcpyAsync(w.point + 2, &one, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    w.h_sys[0].b = w.point;
    w.h_sys[0].x = w.work;
    // CG.solve(in, out, Normal); applyD(out, in, Dagger) (main.cu:456-457)
    int rc = ws_solve(ctx, c, 1, YK_NORMAL, ctx->tol, ctx->tol_mode, ctx->max_iter, ctx->precision, stats);
    if (rc && rc != YK_ENOCONV) return rc;
    YK_CK(launch_dirac(w.work, w.point, C.phi, C.Nt, C.Nx, C.a.m0, C.a.g, C.a.r, 1, YK_FP64, 2, ctx->stream,
                       C.pions ? C.pi : nullptr));
    YK_CK(launch_time_slices_spinor(w.point, w.corr, C.Nt, C.Nx, 2, ctx->stream));
    YK_CK(cudaMemcpyAsync(corr, w.corr, sizeof(double) * C.Nt, cudaMemcpyDeviceToHost, ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return rc;
}

int yk_condensate(yk_ctx* ctx, int c, double* cond, yk_solve_stats* stats)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    Chain& C = ctx->ch[c];
    if (C.a.g == 0.0) {
        *cond = 0.0;   // main.cu:477-481
        if (stats) *stats = yk_solve_stats{0, 0, 0.0, 0.0, 1};
        return YK_OK;
    }
    std::vector<double> F(C.V);
    int rc = YK_OK;
    if (C.pions) {
        // fresh noise: Philox stream kind 3; the sigma force of the pion operator
        rc = pion_solve(ctx, c, 3, nullptr, ctx->precision, stats);
        if (rc && rc != YK_ENOCONV) return rc;
        YK_CK(launch_pion_force(ctx->d_chains + c, C.ws.d_sys, C.n_rhs_pion, C.pi, C.pforce, C.V, ctx->stream));
        YK_CK(cudaMemcpyAsync(F.data(), C.pforce, sizeof(double) * C.V, cudaMemcpyDeviceToHost, ctx->stream));
    } else {
        rc = chain_solve(ctx, c, 3, stats);   // fresh noise: Philox stream kind 3
        if (rc && rc != YK_ENOCONV) return rc;
        StepArgs s = chain_step_args(ctx, c);
        YK_CK(launch_force_drift(s, ctx->d_sys, 1, 1, ctx->stream, ctx->d_state));
        YK_CK(cudaMemcpyAsync(F.data(), C.drift, sizeof(double) * C.V, cudaMemcpyDeviceToHost, ctx->stream));
    }
    YK_CK(cudaStreamSynchronize(ctx->stream));
    double tr = 0.0;
    for (double f : F) tr += f;
    *cond = (tr / C.a.g) / (double)C.V;   // main.cu:473-483
    return rc;
}

int yk_set_eps_bar(yk_ctx* ctx, int c, double eps_bar)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    ctx->h_chains[c].eps_bar = eps_bar;
    ctx->ch[c].a.eps_bar = eps_bar;
    YK_CK(cudaMemcpyAsync(&ctx->d_chains[c].eps_bar, &ctx->h_chains[c].eps_bar, sizeof(double),
                          cudaMemcpyHostToDevice, ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return YK_OK;
}

int yk_get_step(yk_ctx* ctx, int c, int64_t* step)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    YK_CK(cudaMemcpyAsync(step, &ctx->d_chains[c].step, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return YK_OK;
}

int yk_set_time(yk_ctx* ctx, int c, double t)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    ctx->h_chains[c].time = t;
    YK_CK(cudaMemcpyAsync(&ctx->d_chains[c].time, &ctx->h_chains[c].time, sizeof(double), cudaMemcpyHostToDevice,
                          ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return YK_OK;
}

int yk_set_step(yk_ctx* ctx, int c, int64_t step)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    ctx->h_chains[c].step = step;
    YK_CK(cudaMemcpyAsync(&ctx->d_chains[c].step, &ctx->h_chains[c].step, sizeof(int64_t), cudaMemcpyHostToDevice,
                          ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return YK_OK;
}


// ---- learned preconditioner ----

// Relative residual reduction of each inner FP32 solve of the preconditioned
// CG before its FP64 refinement round: YK_PCG_INNER in the environment, else
// 0 (each network times 1e-4 against 1e-5 on its first solves and keeps the
// faster)
static double pcg_inner_tol()
{
    static const double t = [] {
        const char* e = getenv("YK_PCG_INNER");
        const double v = e ? atof(e) : 0.0;
        return v > 0.0 && v < 1.0 ? v : 0.0;
    }();
    return t;
}

static int net_ok(yk_ctx* ctx, int c)
{
    if (int rc = no_pions(ctx, "the learned preconditioner")) return rc;
    if (int rc = chain_ok(ctx, c)) return rc;
    if (!ctx->ch[c].net) {
        set_error("chain %d has no network (yk_net_setup)", c);
        return YK_EINVAL;
    }
    return YK_OK;
}

int yk_net_setup(yk_ctx* ctx, int c, int layers, uint64_t seed, double skip)
{
    if (int rc = chain_ok(ctx, c)) return rc;
    if (int rc = no_pions(ctx, "yk_net_setup")) return rc;
    if (layers < 2 || layers > 8) {
        set_error("yk_net_setup: layers = %d outside [2, 8]", layers);
        return YK_EINVAL;
    }
    Chain& C = ctx->ch[c];
    YK_CK(cudaStreamSynchronize(ctx->stream));
    net_destroy(C.net);
    C.net = nullptr;
    cudaError_t e = cudaSuccess;
    C.net = net_create(C.Nt, C.Nx, layers, &e);
    if (!C.net) {
        set_error("yk_net_setup: %s", cudaGetErrorString(e));
        return YK_ECUDA;
    }
    // small normal weights, 1 / sqrt(fan-in) (splitmix64 + Box-Muller)
    std::vector<float> w((size_t)net_size(C.net));
    uint64_t st = seed;
    auto u01 = [&st]() {
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    if (skip < 0.0) {
        const double d = 4.0 * C.a.r + std::fabs(C.a.m0) + 2.0;
        skip = 1.0 / (d * d);
    }
    net_set_skip(C.net, (float)skip);
    // the last layer starts at 0.1 skip: N(r) ~ 0.1 skip r beside the skip term
    const double scale = 1.0 / std::sqrt(9.0 * 8.0);
    const size_t last = w.size() - 9 * 8 * 4;
    for (size_t i = 0; i < w.size(); ++i) {
        const double a = u01(), b = u01();
        const double f = i >= last && skip != 0.0 ? 0.1 * skip : 1.0;
        w[i] = (float)(f * scale * std::sqrt(-2.0 * std::log(a)) * std::cos(6.283185307179586 * b));
    }
    YK_CK(net_weights(C.net, w.data(), true));
    return YK_OK;
}

int yk_net_size(yk_ctx* ctx, int c)
{
    if (chain_ok(ctx, c) || !ctx->ch[c].net) return 0;
    return net_size(ctx->ch[c].net);
}

int yk_net_weights(yk_ctx* ctx, int c, float* host, int set)
{
    if (int rc = net_ok(ctx, c)) return rc;
    if (!host) {
        set_error("yk_net_weights: host buffer is null");
        return YK_EINVAL;
    }
    YK_CK(cudaStreamSynchronize(ctx->stream));
    YK_CK(net_weights(ctx->ch[c].net, host, set != 0));
    return YK_OK;
}

int yk_net_apply(yk_ctx* ctx, int c, const float* r, float* z)
{
    if (int rc = net_ok(ctx, c)) return rc;
    if (!r || !z) {
        set_error("yk_net_apply: null buffer");
        return YK_EINVAL;
    }
    Chain& C = ctx->ch[c];
    YK_CK(net_forward(C.net, r, C.phi, z, ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return YK_OK;
}

int yk_net_apply_tc(yk_ctx* ctx, int c, const float* r, float* z)
{
    if (int rc = net_ok(ctx, c)) return rc;
    if (!r || !z) {
        set_error("yk_net_apply_tc: null buffer");
        return YK_EINVAL;
    }
    Chain& C = ctx->ch[c];
    YK_CK(net_forward_fast(C.net, r, C.phi, z, ctx->stream));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    return YK_OK;
}

int yk_net_grad(yk_ctx* ctx, int c, const float* r, const float* e, float* grad, double* loss)
{
    if (int rc = net_ok(ctx, c)) return rc;
    if (!r || !e || !grad) {
        set_error("yk_net_grad: null buffer");
        return YK_EINVAL;
    }
    Chain& C = ctx->ch[c];
    double l = 0.0;
    const NetOp op = {C.phi, C.Nt, C.Nx, C.a.m0, C.a.g, C.a.r};
    YK_CK(net_zero_grad(C.net, ctx->stream));
    YK_CK(net_accumulate_grad(C.net, r, e, op, ctx->stream, &l));
    YK_CK(net_grad_to_host(C.net, grad, ctx->stream));
    if (loss) *loss = l;
    return YK_OK;
}

int yk_net_train(yk_ctx* ctx, int c, const yk_net_train_cfg* cfg, yk_net_train_stats* stats)
{
    if (int rc = net_ok(ctx, c)) return rc;
    Chain& C = ctx->ch[c];
    if (!cfg || cfg->n_sources < 1 || cfg->n_levels < 1 || cfg->base_iter < 1 || cfg->steps < 0 ||
        cfg->batch < 1 || !(cfg->lr > 0.0)) {
        set_error("yk_net_train: bad configuration");
        return YK_EINVAL;
    }
    if (C.n_rhs_step == 0) {
        set_error("yk_net_train: chain %d has no fermion systems (g = 0)", c);
        return YK_EINVAL;
    }
    const auto t0 = std::chrono::steady_clock::now();
    SysDev S;
    YK_CK(cudaMemcpy(&S, ctx->d_sys + C.sys0, sizeof(SysDev), cudaMemcpyDeviceToHost));
    const size_t V4 = 4 * (size_t)C.V;
    double* xstar = nullptr;
    YK_CK(cudaMalloc(&xstar, sizeof(double) * V4));
    const int cap = cfg->n_sources * cfg->n_levels;
    const int keep_iter = ctx->max_iter;
    int rc = YK_OK;
    for (int src = 0; src < cfg->n_sources && rc == YK_OK; ++src) {
        const int kind = 100 + src;
        ctx->max_iter = keep_iter;
        rc = chain_solve(ctx, c, kind, nullptr, true);
        if (rc == YK_ENOCONV) rc = YK_OK;
        if (rc) break;
        if (cudaMemcpyAsync(xstar, S.x, sizeof(double) * V4, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess) {
            rc = YK_ECUDA;
            break;
        }
        for (int lv = 0; lv < cfg->n_levels && rc == YK_OK; ++lv) {
            ctx->max_iter = cfg->base_iter << lv;
            rc = chain_solve(ctx, c, kind, nullptr, true);
            if (rc == YK_ENOCONV) rc = YK_OK;
            if (rc) break;
            const cudaError_t e = net_add_pair(C.net, cap, C.phi, C.a.m0, C.a.g, C.a.r, S.b, xstar, S.x, ctx->stream);
            if (e != cudaSuccess && e != cudaErrorInvalidValue) rc = YK_ECUDA;   // a vanished error adds no pair
        }
    }
    ctx->max_iter = keep_iter;
    cudaFree(xstar);
    if (rc) return rc;
    yk_net_train_stats out = {};
    out.pairs = net_pairs(C.net);
    const NetOp op = {C.phi, C.Nt, C.Nx, C.a.m0, C.a.g, C.a.r};
    YK_CK(net_mean_loss(C.net, op, ctx->stream, &out.loss0));
    YK_CK(net_train(C.net, op, cfg->steps, cfg->batch, (float)cfg->lr, cfg->seed, ctx->stream));
    YK_CK(net_mean_loss(C.net, op, ctx->stream, &out.loss1));
    out.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = out;
    return YK_OK;
}

int yk_fgcr_solve(yk_ctx* ctx, int c, const double* b, double* x, double tol, int tol_mode, int max_iter, int use_net,
                  yk_solve_stats* stats)
{
    if (int rc = net_ok(ctx, c)) return rc;
    if (!b || !x || b == x || max_iter < 0 || !(tol >= 0.0) || (tol_mode != YK_TOL_ABS && tol_mode != YK_TOL_REL)) {
        set_error("yk_fgcr_solve: bad arguments");
        return YK_EINVAL;
    }
    Chain& C = ctx->ch[c];
    FgcrResult r = {};
    YK_CK(fgcr_solve(C.net, use_net != 0, C.phi, C.a.m0, C.a.g, C.a.r, b, x, tol, tol_mode, max_iter, 16, 1e-4,
                     ctx->stream, &r));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    if (stats) *stats = yk_solve_stats{r.iterations, r.outer, r.rr, r.rr0, r.converged};
    if (!r.converged) {
        set_error("yk_fgcr_solve: %d iterations, |r|^2 = %g > the tolerance", r.iterations, r.rr);
        return YK_ENOCONV;
    }
    return YK_OK;
}

int yk_autotune(yk_ctx* ctx, yk_tune_result* out)
{
    if (int rc = no_pions(ctx, "yk_autotune")) return rc;
    if (!ctx) {
        set_error("yk_autotune: null context");
        return YK_EINVAL;
    }
    if (ctx->gexec) {   // captured with the previous choice
        YK_CK(cudaStreamSynchronize(ctx->stream));
        cudaGraphExecDestroy(ctx->gexec);
        ctx->gexec = nullptr;
    }
    for (auto& g : ctx->io) cudaGraphExecDestroy(g.exec);
    ctx->io.clear();
    if (int rc = run_autotune(ctx)) return rc;
    if (out) *out = ctx->tune;
    return YK_OK;
}

int yk_tune_report(yk_ctx* ctx, yk_tune_result* out)
{
    if (!ctx || !out) {
        set_error("yk_tune_report: bad arguments");
        return YK_EINVAL;
    }
    *out = ctx->tune;
    for (const Chain& C : ctx->ch)
        if (C.net) {
            net_tile(C.net, &out->conv_rows, &out->conv_cols, &out->conv_layers_per_launch);
            out->pcg_inner_tol = pcg_inner_choice(C.net);
            break;
        }
    return YK_OK;
}

int yk_langevin_step_learned(yk_ctx* ctx, int n_steps, int use_net, yk_solve_stats* stats)
{
    if (int rc = no_pions(ctx, "yk_langevin_step_learned")) return rc;
    if (!ctx || n_steps < 0) {
        set_error("yk_langevin_step_learned: bad arguments");
        return YK_EINVAL;
    }
    for (size_t c = 0; c < ctx->ch.size(); ++c)
        if (use_net && ctx->ch[c].n_rhs_step > 0 && !ctx->ch[c].net) {
            set_error("yk_langevin_step_learned: chain %zu has no network (yk_net_setup)", c);
            return YK_EINVAL;
        }
    std::vector<SysDev> sys(ctx->nsys);
    std::vector<CGState> st(ctx->nsys);
    if (ctx->nsys > 0)
        YK_CK(cudaMemcpy(sys.data(), ctx->d_sys, sizeof(SysDev) * ctx->nsys, cudaMemcpyDeviceToHost));
    yk_solve_stats tot = {0, 0, 0.0, 0.0, 1};
    NoiseTables nt = {ctx->d_rows, ctx->nrows, ctx->d_cols, ctx->ncols, ctx->d_white, ctx->nwhite};
    for (int i = 0; i < n_steps; ++i) {
        YK_CK(launch_noise_tables(ctx->d_chains, nt, ctx->max_nx, ctx->max_cols, nullptr, ctx->stream));
        for (Chain& C : ctx->ch) {
            if (C.n_rhs_step == 0) continue;
            // the step's sources (Philox stream 2 at the chain's step), as the CG would draw them
            YK_CK(launch_eta(ctx->d_sys, ctx->d_sys_tiles + C.cg_tile0, C.cg_tile1 - C.cg_tile0, 2, ctx->stream));
            for (int j = 0; j < C.n_rhs_step; ++j) {
                LearnedNet* net = C.net ? C.net : C.pcg_ws;
                if (!net) {   // identity preconditioner: an unused network provides the solver's buffers
                    cudaError_t e = cudaSuccess;
                    net = C.pcg_ws = net_create(C.Nt, C.Nx, 2, &e);
                    if (!net) {
                        set_error("yk_langevin_step_learned: %s", cudaGetErrorString(e));
                        return YK_ECUDA;
                    }
                }
                const SysDev& S = sys[C.sys0 + j];
                FgcrResult r = {};
                YK_CK(pcg_solve(net, use_net != 0, C.phi, C.a.m0, C.a.g, C.a.r, S.b, S.x, ctx->tol, ctx->tol_mode,
                                ctx->max_iter, pcg_inner_tol(), ctx->stream, &r));
                CGState& q = st[C.sys0 + j];
                std::memset(&q, 0, sizeof(q));
                q.rr = r.rr;
                q.rr0 = r.rr0;
                q.iters = r.iterations;
                q.converged = r.converged;
                q.status = r.converged ? 0 : YK_ENOCONV;
                q.n_ru = r.outer;
                tot.iterations += r.iterations;
                tot.reliable_updates += r.outer;
                tot.rr += r.rr;
                tot.rr0 += r.rr0;
                if (!r.converged) tot.converged = 0;
            }
        }
        if (ctx->nsys > 0)
            YK_CK(cudaMemcpyAsync(ctx->d_state, st.data(), sizeof(CGState) * ctx->nsys, cudaMemcpyHostToDevice,
                                  ctx->stream));
        StepArgs s = step_args(ctx);
        YK_CK(launch_force_drift(s, ctx->d_sys, 0, 1, ctx->stream, nullptr));
        YK_CK(launch_update(s, ctx->d_state, ctx->stream));
        // st is reused by the next step: its copy must have left the host
        YK_CK(cudaStreamSynchronize(ctx->stream));
    }
    if (stats) *stats = tot;
    return YK_OK;
}

int yk_pcg_solve(yk_ctx* ctx, int c, const double* b, double* x, double tol, int tol_mode, int max_iter, int use_net,
                 yk_solve_stats* stats)
{
    if (int rc = net_ok(ctx, c)) return rc;
    if (!b || !x || b == x || max_iter < 0 || !(tol >= 0.0) || (tol_mode != YK_TOL_ABS && tol_mode != YK_TOL_REL)) {
        set_error("yk_pcg_solve: bad arguments");
        return YK_EINVAL;
    }
    Chain& C = ctx->ch[c];
    FgcrResult r = {};
    YK_CK(pcg_solve(C.net, use_net != 0, C.phi, C.a.m0, C.a.g, C.a.r, b, x, tol, tol_mode, max_iter, pcg_inner_tol(),
                    ctx->stream, &r));
    YK_CK(cudaStreamSynchronize(ctx->stream));
    if (stats) *stats = yk_solve_stats{r.iterations, r.outer, r.rr, r.rr0, r.converged};
    if (!r.converged) {
        set_error("yk_pcg_solve: %d iterations, |r|^2 = %g > the tolerance", r.iterations, r.rr);
        return YK_ENOCONV;
    }
    return YK_OK;
}

}  // extern "C"
