// yk_noalloc.cu -- yk_cg_solve_static: the FP64 CG solve of yk_cg_solve
// (CGsolver::solve, code/src/CGsolver.cu:42-59) without a context and without
// any device allocation.  Its scratch -- the CG vectors r and p (two each),
// D p and A p, the per-tile partial sums, the tile table, the system record,
// the solver state and coefficients, the grid barrier, the neighbour flags
// and the error flags -- lives in one
// file-scope device array of fixed size, so lattices up to
// kStaticMaxSites sites are accepted and larger ones are refused.
//
// Nothing in the array has to start at zero: the preparation kernel that
// launch_cg runs before every solve resets the barrier, the error flag and
// the solver state, the setup kernel below writes the system record and the
// tile table, and the CG kernel writes every vector before reading it.
//
// Calls that overlap in time (on different streams or host threads) share
// the one array and race; callers serialise them.
#include <mutex>

#include "yk_common.cuh"
#include "yk_host.h"
#include "yk_kernels.h"

namespace yk {

namespace {

constexpr int kStaticMaxSites = 16384;                      // e.g. 128 x 128
constexpr int kStaticMaxTiles = kStaticMaxSites / kTile;    // 64
constexpr size_t kAlign = 256;
constexpr size_t up(size_t n) { return (n + kAlign - 1) / kAlign * kAlign; }

// byte offsets of the pieces inside the array
constexpr size_t kVecBytes = sizeof(double) * 8 * kStaticMaxSites;   // one FP64 complex spinor field
constexpr size_t oR0 = 0;
constexpr size_t oR1 = oR0 + kVecBytes;
constexpr size_t oP0 = oR1 + kVecBytes;
constexpr size_t oP1 = oP0 + kVecBytes;
constexpr size_t oT = oP1 + kVecBytes;
constexpr size_t oAp = oT + kVecBytes;
constexpr size_t oPartial = oAp + kVecBytes;
constexpr size_t oTiles = oPartial + up(sizeof(Partial) * kStaticMaxTiles);
constexpr size_t oSys = oTiles + up(sizeof(int2) * kStaticMaxTiles);
constexpr size_t oState = oSys + up(sizeof(SysDev));
constexpr size_t oCoef = oState + up(sizeof(CGState));
constexpr size_t oBar = oCoef + up(sizeof(CGCoef));
constexpr size_t oNbr = oBar + up(sizeof(GridBarrier));
constexpr size_t oFlags = oNbr + up(sizeof(unsigned) * kFlagStride * kMaxGrid);
constexpr size_t kStaticScratchBytes = oFlags + up(sizeof(int) * 4);   // about 6.6 MB

static __device__ __align__(256) unsigned char g_cg_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned char* g_base[kMaxDevices] = {};
unsigned long long g_ctx_id[kMaxDevices] = {};   // context the address of g_base[dev] belongs to

// Unique id of the calling thread's current context (0 if unavailable).  A
// cudaDeviceReset() ends the device's primary context; the module is loaded
// again into the next one, possibly at another address, and that context has
// a new id.  The driver functions are reached through the runtime, so the
// library needs no link against libcuda.
unsigned long long current_context_id()
{
    typedef int (*CtxGetCurrent)(void**);
    typedef int (*CtxGetId)(void*, unsigned long long*);
    static CtxGetCurrent get_current = nullptr;
    static CtxGetId get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetId>(f);
        looked_up = true;
    }
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

// The system record and tile table of one lattice, written on the device.
__global__ void static_setup_kernel(unsigned char* base, const double* sigma, const double* b, double* x, int Nt,
                                    int Nx, double m0, double g, double r)
{
    const int V = Nt * Nx, nt = (V + kTile - 1) / kTile;
    int2* tiles = reinterpret_cast<int2*>(base + oTiles);
    for (int t = threadIdx.x; t < nt; t += blockDim.x) tiles[t] = make_int2(0, t * kTile);
    if (threadIdx.x == 0) {
        SysDev S;
        memset(&S, 0, sizeof(S));
        S.chain = 0;
        S.rhs = 0;
        S.Nt = Nt;
        S.Nx = Nx;
        S.V = V;
        S.tile0 = 0;
        S.ntiles = nt;
        S.m0 = m0;
        S.g = g;
        S.r = r;
        S.sigma = sigma;
        S.b = const_cast<double*>(b);
        S.x = x;
        S.r64[0] = reinterpret_cast<double*>(base + oR0);
        S.r64[1] = reinterpret_cast<double*>(base + oR1);
        S.p64[0] = reinterpret_cast<double*>(base + oP0);
        S.p64[1] = reinterpret_cast<double*>(base + oP1);
        S.t64 = reinterpret_cast<double*>(base + oT);
        S.Ap64 = reinterpret_cast<double*>(base + oAp);
        S.gen_eta = 0;
        *reinterpret_cast<SysDev*>(base + oSys) = S;
    }
}

// Device address of the array on the current device: looked up once per device
// and again after the device's context changed (a cudaDeviceReset).
int scratch_base(unsigned char** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_error("yk_cg_solve_static: cudaGetDevice failed: %s", cudaGetErrorString(e));
        return YK_ECUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("yk_cg_solve_static: device %d beyond the %d supported", dev, kMaxDevices);
        return YK_EINVAL;
    }
    // makes the device's primary context current (creating it if a reset ended it)
    e = cudaSetDevice(dev);
    if (e != cudaSuccess) {
        set_error("yk_cg_solve_static: cudaSetDevice failed: %s", cudaGetErrorString(e));
        return YK_ECUDA;
    }
    const unsigned long long ctx_id = current_context_id();
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_base[dev] || ctx_id != g_ctx_id[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_cg_scratch);
        if (e != cudaSuccess || !p) {
            set_error("yk_cg_solve_static: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return YK_ECUDA;
        }
        g_base[dev] = static_cast<unsigned char*>(p);
        g_ctx_id[dev] = ctx_id;
    }
    *out = g_base[dev];
    return YK_OK;
}

}  // namespace

}  // namespace yk

using namespace yk;

extern "C" int yk_cg_solve_static(const double* sigma, int Nt, int Nx, double m0, double g, double r, const void* b,
                                  void* x, int mtype, double tol, int tol_mode, int max_iter, void* stream,
                                  yk_solve_stats* stats)
{
    if (!sigma || !b || !x || b == x || Nt < 2 || Nx < 2 || max_iter < 0 || max_iter > 1000000 ||
        (mtype != YK_NORMAL && mtype != YK_DAGGER) || (tol_mode != YK_TOL_ABS && tol_mode != YK_TOL_REL) ||
        !(tol >= 0.0)) {
        set_error("yk_cg_solve_static: bad arguments");
        return YK_EINVAL;
    }
    if ((int64_t)Nt * Nx > kStaticMaxSites) {
        set_error("yk_cg_solve_static: lattice %dx%d has %lld sites, more than the %d of the static scratch", Nt, Nx,
                  (long long)Nt * Nx, kStaticMaxSites);
        return YK_EINVAL;
    }
    unsigned char* base = nullptr;
    if (int rc = scratch_base(&base)) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    static_setup_kernel<<<1, 64, 0, s>>>(base, sigma, static_cast<const double*>(b), static_cast<double*>(x), Nt, Nx,
                                         m0, g, r);
    cudaError_t e = cudaGetLastError();
    CGArgs a = {};
    a.sys = reinterpret_cast<SysDev*>(base + oSys);
    a.sys_first = 0;
    a.sys_count = 1;
    a.tiles = reinterpret_cast<const int2*>(base + oTiles);
    a.tile_begin = 0;
    a.tile_end = (Nt * Nx + kTile - 1) / kTile;
    a.eta_kind = 0;
    a.st = reinterpret_cast<CGState*>(base + oState);
    a.partial = reinterpret_cast<Partial*>(base + oPartial);
    a.coef = reinterpret_cast<CGCoef*>(base + oCoef);
    a.flags = reinterpret_cast<unsigned*>(base + oNbr);
    a.bar = reinterpret_cast<GridBarrier*>(base + oBar);
    a.err = reinterpret_cast<int*>(base + oFlags);
    a.n_active = a.err + 1;
    a.any_ru = a.err + 2;
    a.max_iter = max_iter;
    a.mtype = mtype;
    a.tol_mode = tol_mode;
    a.tol = tol;
    a.reliable_every = 0;
    a.reliable_delta = 0.1;
    if (e == cudaSuccess) e = launch_cg(a, 2, false, s, nullptr);
    CGState st = {};
    int err = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st, a.st, sizeof(st), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&err, a.err, sizeof(err), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_error("yk_cg_solve_static: %s", cudaGetErrorString(e));
        return YK_ECUDA;
    }
    if (err) {
        set_error("yk_cg_solve_static: a bounded device wait gave up (status %d)", err);
        return YK_ETIMEOUT;
    }
    yk_solve_stats out = {};
    out.iterations = st.iters;
    out.reliable_updates = 0;
    out.rr = st.rr;
    out.rr0 = st.rr0;
    out.converged = st.converged;
    if (stats) *stats = out;
    if (st.status) {
        set_error("yk_cg_solve_static: status %d after %d iterations (|r|^2 = %g)", st.status, st.iters, st.rr);
        return st.status;
    }
    return YK_OK;
}
