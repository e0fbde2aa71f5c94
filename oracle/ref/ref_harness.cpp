// ref_harness.cpp -- runs the reference's own CUDA kernels on injected inputs
// and dumps inputs and outputs as golden vectors.
//
// TEST INFRASTRUCTURE ONLY.  The device code is the reference's, compiled from
// its sources by oracle/ref/build_ref.py into oracle/_ref/ref_<Nt>x<Nx>.fatbin;
// this host program replaces code/src/main.cu (which needs the absent toml11
// header): it loads the fatbin with the CUDA driver API, sets the reference's
// __constant__ parameters (main.cu:268-278), builds the neighbour tables
// (Dirac.cu:10-21) and the Laplacian CSR (Laplace.cu:61-100), sizes every
// cooperative launch by occupancy as the reference does (Dirac.cu:25-34,
// CGsolver.cu:44-58, device_info.h:36-62), calls cuFFT exactly as
// colouredNoise.cpp:88-94, 155-178 does, and writes every array to a binary
// dump read by oracle/ref/make_golden.py.
//
// Usage: ref_harness <fatbin> <symbols.txt> <Nt> <Nx> <out.bin>
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#define CK(x)                                                                                   \
    do {                                                                                        \
        CUresult r_ = (x);                                                                      \
        if (r_ != CUDA_SUCCESS) {                                                               \
            const char* s_ = nullptr;                                                           \
            cuGetErrorString(r_, &s_);                                                          \
            std::fprintf(stderr, "%s:%d %s -> %s\n", __FILE__, __LINE__, #x, s_ ? s_ : "?");    \
            std::exit(2);                                                                       \
        }                                                                                       \
    } while (0)
#define CF(x)                                                                                   \
    do {                                                                                        \
        cufftResult r_ = (x);                                                                   \
        if (r_ != CUFFT_SUCCESS) {                                                              \
            std::fprintf(stderr, "%s:%d %s -> cufft %d\n", __FILE__, __LINE__, #x, (int)r_);    \
            std::exit(3);                                                                       \
        }                                                                                       \
    } while (0)

static int Nt, Nx, V;
static CUmodule mod;
static std::map<std::string, CUfunction> fns;
static FILE* dump;

// ------------------------------------------------------------ inputs
static uint64_t rng_state = 0x9E3779B97F4A7C15ULL;
static double uni01()
{
    uint64_t z = (rng_state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return ((z >> 11) + 0.5) * 0x1p-53;
}
static double unif() { return 2.0 * uni01() - 1.0; }
static double gauss() { return std::sqrt(-2.0 * std::log(uni01())) * std::cos(2.0 * M_PI * uni01()); }

static void put(const char* name, const std::vector<double>& v)
{
    char nm[32] = {0};
    std::strncpy(nm, name, 31);
    const int64_t n = (int64_t)v.size();
    std::fwrite(nm, 1, 32, dump);
    std::fwrite(&n, sizeof n, 1, dump);
    std::fwrite(v.data(), sizeof(double), v.size(), dump);
}

// ------------------------------------------------------------ device helpers
static CUdeviceptr dalloc(size_t bytes)
{
    CUdeviceptr p;
    CK(cuMemAlloc(&p, bytes));
    CK(cuMemsetD8(p, 0, bytes));
    return p;
}
static void h2d(CUdeviceptr d, const void* h, size_t bytes) { CK(cuMemcpyHtoD(d, h, bytes)); }
static std::vector<double> d2h(CUdeviceptr d, size_t n)
{
    std::vector<double> v(n);
    CK(cuMemcpyDtoH(v.data(), d, n * sizeof(double)));
    return v;
}
template <typename T>
static void set_const(const char* name, T v)
{
    CUdeviceptr p;
    size_t b;
    CK(cuModuleGetGlobal(&p, &b, mod, name));
    CK(cuMemcpyHtoD(p, &v, sizeof(T)));
}

// Occupancy-sized cooperative launch (cudaOccupancyMaxPotentialBlockSize).
static void coop(const char* k, void** args, int smem_per_warp_bytes = 0, int fixed_smem = 0)
{
    CUfunction f = fns.at(k);
    int min_grid = 0, block = 0;
    CK(cuOccupancyMaxPotentialBlockSize(&min_grid, &block, f, nullptr, 0, 0));
    const unsigned smem = (unsigned)(fixed_smem + smem_per_warp_bytes * (block / 32));
    CK(cuLaunchCooperativeKernel(f, min_grid, 1, 1, block, 1, 1, smem, nullptr, args));
    CK(cuCtxSynchronize());
}

// KernelLaunchInfo (device_info.h:36-62) restated.
struct Kli {
    int blocks, threads;
};
static Kli kli(const char* k)
{
    CUfunction f = fns.at(k);
    CUdevice dev;
    CK(cuCtxGetDevice(&dev));
    int sms, maxtpsm, maxtpb;
    CK(cuDeviceGetAttribute(&sms, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, dev));
    CK(cuDeviceGetAttribute(&maxtpsm, CU_DEVICE_ATTRIBUTE_MAX_THREADS_PER_MULTIPROCESSOR, dev));
    CK(cuDeviceGetAttribute(&maxtpb, CU_DEVICE_ATTRIBUTE_MAX_THREADS_PER_BLOCK, dev));
    int nb = 0, nt = 0;
    CK(cuOccupancyMaxPotentialBlockSize(&nb, &nt, f, nullptr, 0, 0));
    const int maxBlocks = sms * (maxtpsm / maxtpb);
    nt = std::min(nt, V);
    nb = std::min(nb, maxBlocks);
    nb = std::min(V / nt, nb);
    nb = std::max(nb, 1);
    int per = 0;
    CK(cuOccupancyMaxActiveBlocksPerMultiprocessor(&per, f, nt, nt * sizeof(double)));
    if (nb > per * sms) nb = per * sms;
    return {nb, nt};
}
static void coop_kli(const char* k, const Kli& g, void** args, unsigned smem)
{
    CK(cuLaunchCooperativeKernel(fns.at(k), g.blocks, 1, 1, g.threads, 1, 1, smem, nullptr, args));
    CK(cuCtxSynchronize());
}

// ------------------------------------------------------------ reference objects
struct Tables {
    CUdeviceptr iup, idn, I, J, vals;
};
static Tables make_tables()
{
    // Dirac.cu:10-21 (indices premultiplied by 4)
    std::vector<int> iup(2 * V), idn(2 * V);
    for (int i = 0; i < V; ++i) {
        const int t = i / Nx, x = i % Nx;
        iup[2 * i + 0] = 4 * (((t + 1) % Nt) * Nx + x);
        iup[2 * i + 1] = 4 * (t * Nx + (x + 1) % Nx);
        idn[2 * i + 0] = 4 * (((t - 1 + Nt) % Nt) * Nx + x);
        idn[2 * i + 1] = 4 * (t * Nx + (x - 1 + Nx) % Nx);
    }
    // Laplace.cu:61-100: sorted columns, -2d on the diagonal, 1 elsewhere
    std::vector<int> I(V + 1), J(5 * V);
    std::vector<double> vals(5 * V);
    for (int r = 0; r < V; ++r) {
        const int t = r / Nx, x = r % Nx;
        std::array<int, 5> c = {r, ((t + 1) % Nt) * Nx + x, ((t - 1 + Nt) % Nt) * Nx + x, t * Nx + (x + 1) % Nx,
                                t * Nx + (x - 1 + Nx) % Nx};
        std::sort(c.begin(), c.end());
        for (int j = 0; j < 5; ++j) {
            J[5 * r + j] = c[j];
            vals[5 * r + j] = (c[j] != r) ? 1.0 : -4.0;
        }
        I[r + 1] = 5 * (r + 1);
    }
    Tables T;
    T.iup = dalloc(sizeof(int) * 2 * V);
    T.idn = dalloc(sizeof(int) * 2 * V);
    T.I = dalloc(sizeof(int) * (V + 1));
    T.J = dalloc(sizeof(int) * 5 * V);
    T.vals = dalloc(sizeof(double) * 5 * V);
    h2d(T.iup, iup.data(), sizeof(int) * 2 * V);
    h2d(T.idn, idn.data(), sizeof(int) * 2 * V);
    h2d(T.I, I.data(), sizeof(int) * (V + 1));
    h2d(T.J, J.data(), sizeof(int) * 5 * V);
    h2d(T.vals, vals.data(), sizeof(double) * 5 * V);
    return T;
}

static void set_params(double m2, double lam, double g, double m0, double r, double cut, int drift_mode,
                       double eps_bar)
{
    set_const("m2", m2);
    set_const("lambda", lam);
    set_const("epsBar", eps_bar);
    set_const("yukawa_coupling_gpu", g);
    set_const("fermion_mass_gpu", m0);
    const double im[2] = {0.0, 1.0};
    CUdeviceptr p;
    size_t b;
    CK(cuModuleGetGlobal(&p, &b, mod, "im_gpu"));
    CK(cuMemcpyHtoD(p, im, sizeof im));
    set_const("cutFraction_gpu", cut);
    set_const("sq2Kappa_gpu", 1.0);
    set_const("driftMode_gpu", drift_mode);
    set_const("WilsonParam_gpu", r);
}

static void applyD(CUdeviceptr in, CUdeviceptr out, int dagger, CUdeviceptr M, const Tables& T)
{
    CUdeviceptr tin = in, tout = out, tm = M, ti = T.iup, td = T.idn;
    int mt = dagger;
    void* args[] = {&tin, &tout, &mt, &tm, &ti, &td};
    coop("applyD_gpu", args);
}

struct CGBufs {
    CUdeviceptr temp, temp2, r, p, alpha, beta, dot, rmodsq;
};
static CGBufs make_cg()
{
    const size_t s = 16 * 4 * (size_t)V;
    return {dalloc(s), dalloc(s), dalloc(s), dalloc(s), dalloc(16), dalloc(16), dalloc(16), dalloc(8)};
}
static void cg_solve(CUdeviceptr in, CUdeviceptr out, int mtype, CUdeviceptr M, const Tables& T, CGBufs& B)
{
    CUdeviceptr a0 = in, a1 = out, a2 = B.temp, a3 = B.temp2, a4 = B.r, a5 = B.p, a6 = B.alpha, a7 = B.beta,
                a8 = M, a9 = T.iup, a10 = T.idn, a12 = B.dot, a13 = B.rmodsq;
    int mt = mtype;
    void* args[] = {&a0, &a1, &a2, &a3, &a4, &a5, &a6, &a7, &a8, &a9, &a10, &mt, &a12, &a13};
    // One block of one warp.  With the occupancy-sized grid of CGsolver.cu:44-58
    // the kernel races: thread 0 of block 0 negates *alpha (CGsolver.cu:146)
    // with no grid sync after the x update that reads *alpha (:143), so other
    // blocks can apply -alpha to x.  In a single warp every lane reads *alpha
    // before lane 0 negates it; the kernel's arithmetic is unchanged.
    CK(cuLaunchCooperativeKernel(fns.at("solve_kernel"), 1, 1, 1, 32, 1, 1, 16, nullptr, args));
    CK(cuCtxSynchronize());
}

// The same solve with the reference's own occupancy-sized launch (racy x).
static void cg_solve_occupancy(CUdeviceptr in, CUdeviceptr out, int mtype, CUdeviceptr M, const Tables& T,
                               CGBufs& B)
{
    CUdeviceptr a0 = in, a1 = out, a2 = B.temp, a3 = B.temp2, a4 = B.r, a5 = B.p, a6 = B.alpha, a7 = B.beta,
                a8 = M, a9 = T.iup, a10 = T.idn, a12 = B.dot, a13 = B.rmodsq;
    int mt = mtype;
    void* args[] = {&a0, &a1, &a2, &a3, &a4, &a5, &a6, &a7, &a8, &a9, &a10, &mt, &a12, &a13};
    coop("solve_kernel", args, 16);   // smem = sizeof(complex<double>) * (threads / 32)
}

static std::vector<double> mask_half(double cut)
{
    // colouredNoise.cpp:16-29, 138-145 (host code of the ColouredNoise constructor)
    const double momentumCut = std::sqrt(2.0) * M_PI * cut;
    const double cutSq = momentumCut * momentumCut;
    std::vector<double> m;
    const int sizes[2] = {Nt, Nx};
    for (int pos = 0; pos < V; ++pos) {
        int coo[2] = {pos / Nx, pos % Nx};
        double msq = 0.0, sgn = 1.0;
        if (coo[1] > std::floor(Nx / 2)) sgn = -1.0;
        for (int n = 0; n < 2; ++n) {
            const int L = sizes[n];
            const double tmp = (coo[n] <= std::floor(L / 2) ? coo[n] : coo[n] - L) * 2.0 * M_PI / L;
            msq += tmp * tmp;
        }
        msq *= sgn;
        if (msq >= 0) m.push_back(msq <= cutSq ? 1.0 / V : 0.0);
    }
    return m;
}

static std::vector<double> coloured(const std::vector<double>& w, double cut)
{
    const int nfreq = Nt * (Nx / 2 + 1);
    CUdeviceptr dw = dalloc(8 * (size_t)V), dtmp = dalloc(16 * (size_t)nfreq), dm = dalloc(8 * (size_t)nfreq);
    h2d(dw, w.data(), 8 * (size_t)V);
    const std::vector<double> m = mask_half(cut);
    h2d(dm, m.data(), 8 * m.size());
    int sizes[2] = {Nt, Nx};
    cufftHandle pf, pr;
    CF(cufftPlanMany(&pf, 2, sizes, NULL, 1, V, NULL, 1, V, CUFFT_D2Z, 1));
    CF(cufftPlanMany(&pr, 2, sizes, NULL, 1, V, NULL, 1, V, CUFFT_Z2D, 1));
    CF(cufftExecD2Z(pf, (cufftDoubleReal*)dw, (cufftDoubleComplex*)dtmp));
    CK(cuCtxSynchronize());
    const Kli g = kli("ApplyMask");
    CUdeviceptr a0 = dtmp, a1 = dm;
    int n = V;
    void* args[] = {&a0, &a1, &n};
    coop_kli("ApplyMask", g, args, 0);
    CF(cufftExecZ2D(pr, (cufftDoubleComplex*)dtmp, (cufftDoubleReal*)dw));
    CK(cuCtxSynchronize());
    cufftDestroy(pf);
    cufftDestroy(pr);
    std::vector<double> xi = d2h(dw, V);
    cuMemFree(dw);
    cuMemFree(dtmp);
    cuMemFree(dm);
    return xi;
}

// getForce with an injected eta (FermionicDrift.cu:57-80, skipping fillNormalRND)
static std::vector<double> force(CUdeviceptr eta, CUdeviceptr M, const Tables& T, CGBufs& B)
{
    CUdeviceptr buf = dalloc(64 * (size_t)V), after = dalloc(64 * (size_t)V), F = dalloc(8 * (size_t)V);
    cg_solve(eta, buf, 1, M, T, B);
    applyD(buf, after, 0, M, T);
    CUdeviceptr a0 = after, a1 = eta, a2 = F;
    void* args[] = {&a0, &a1, &a2};
    coop("computeDrift", args);
    std::vector<double> out = d2h(F, V);
    cuMemFree(buf);
    cuMemFree(after);
    cuMemFree(F);
    return out;
}

// Run kernel (langevin_gpu_v2.cu:65-118) with drift preset to the fermion force.
static double run_update(CUdeviceptr phi, CUdeviceptr drift, CUdeviceptr noise, const Tables& T, double eps_bar,
                         double* maxdrift)
{
    CUdeviceptr eps = dalloc(8), md = dalloc(8);
    h2d(eps, &eps_bar, 8);
    const Kli g = kli("Run");
    double export_time = 1.0;
    int n = V;
    CUdeviceptr a0 = eps, a2 = phi, a3 = drift, a4 = noise, a6 = T.I, a7 = T.J, a8 = T.vals, a9 = md;
    void* args[] = {&a0, &export_time, &a2, &a3, &a4, &n, &a6, &a7, &a8, &a9};
    coop_kli("Run", g, args, (unsigned)(sizeof(double) * std::max(g.threads, 32)));
    const double e = d2h(eps, 1)[0];
    *maxdrift = d2h(md, 1)[0];
    cuMemFree(eps);
    cuMemFree(md);
    return e;
}

// ------------------------------------------------------------ timing
static std::vector<double> read_raw(const char* path, size_t n)
{
    std::vector<double> v(n);
    FILE* f = std::fopen(path, "rb");
    if (!f || std::fread(v.data(), sizeof(double), n, f) != n) {
        std::fprintf(stderr, "cannot read %zu doubles from %s\n", n, path);
        std::exit(5);
    }
    std::fclose(f);
    return v;
}

static double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Times the reference's own kernels on this GPU, launched and synchronised as
// the reference launches them: the Dirac apply (Dirac.cu:23-35), the CG solve
// of a given right-hand side (CGsolver.cu:42-59, its occupancy-sized grid)
// and full Langevin steps (main.cu:370-381: ColouredNoise::operator() with
// DoRNG, cuFFT and ApplyMask, colouredNoise.cpp:155-178; getForce with
// fillNormalRND, setZero_kernel, the solve, applyD and computeDrift,
// FermionicDrift.cu:57-80; Run; the eps copy to the host), from the given
// field.  Vectors live in device memory (the reference allocates managed
// memory).  Writes one JSON object.
static int time_mode(const char* field_path, const char* b_path, int steps, const char* out_path)
{
    const double m2 = -0.5, lam = 1.0, g = 0.5, m0 = 0.1, eps_bar = 0.01, cut = 0.35355339059327373;
    set_params(m2, lam, g, m0, 1.0, cut, 0, eps_bar);
    const Tables T = make_tables();
    CGBufs B = make_cg();
    const size_t SB = 64 * (size_t)V;
    CUdeviceptr phi = dalloc(8 * (size_t)V), bvec = dalloc(SB), x = dalloc(SB), y = dalloc(SB);
    const std::vector<double> f0 = read_raw(field_path, V), b = read_raw(b_path, 8 * (size_t)V);
    h2d(phi, f0.data(), 8 * (size_t)V);
    h2d(bvec, b.data(), SB);
    CUevent e0, e1;
    CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
    CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
    auto timed = [&](auto&& fn, int reps) {
        fn();   // warm-up
        float tot = 0.f;
        for (int i = 0; i < reps; ++i) {
            CK(cuEventRecord(e0, nullptr));
            fn();
            CK(cuEventRecord(e1, nullptr));
            CK(cuEventSynchronize(e1));
            float ms = 0.f;
            CK(cuEventElapsedTime(&ms, e0, e1));
            tot += ms;
        }
        return tot / reps;
    };
    // Dirac apply: occupancy query, cooperative launch, synchronisation
    const float ms_dirac = timed([&] { applyD(bvec, y, 0, phi, T); }, 20);
    // CG on D^dag D with the reference's grid (tolerance 1e-8 absolute, 1000 iterations)
    const float ms_cg = timed([&] { cg_solve_occupancy(bvec, x, 1, phi, T, B); }, 5);
    // full steps
    const Kli kr = kli("Run");
    CUdeviceptr states_noise = dalloc(64 * (size_t)kr.blocks * kr.threads);
    // fillNormalRND reads state[thread rank] of its whole occupancy-sized grid
    // (FermionicDrift.cu:104) before its loop over the 4V states, so the
    // buffer holds max(4V, grid threads) states (64 bytes each, more than a
    // curandStateXORWOW's 48)
    int rnd_grid = 0, rnd_block = 0;
    CK(cuOccupancyMaxPotentialBlockSize(&rnd_grid, &rnd_block, fns.at("fillNormalRND"), nullptr, 0, 0));
    const size_t n_states_f = std::max((size_t)4 * V, (size_t)rnd_grid * rnd_block);
    CUdeviceptr states_f = dalloc(64 * n_states_f);
    int seed = 1234, svol = 4 * V;
    {
        CUdeviceptr a1 = states_noise;
        void* args[] = {&seed, &a1};
        coop_kli("setup_kernel", kr, args, 0);
        CUdeviceptr b1 = states_f;
        void* args2[] = {&seed, &b1, &svol};
        coop("random_setup_kernel", args2);
    }
    const int nfreq = Nt * (Nx / 2 + 1);
    CUdeviceptr noise = dalloc(8 * (size_t)V), tmp = dalloc(16 * (size_t)nfreq), mask = dalloc(8 * (size_t)nfreq);
    const std::vector<double> mk = mask_half(cut);
    h2d(mask, mk.data(), 8 * mk.size());
    int sizes[2] = {Nt, Nx};
    cufftHandle pf, pr;
    CF(cufftPlanMany(&pf, 2, sizes, NULL, 1, V, NULL, 1, V, CUFFT_D2Z, 1));
    CF(cufftPlanMany(&pr, 2, sizes, NULL, 1, V, NULL, 1, V, CUFFT_Z2D, 1));
    CUdeviceptr eta = dalloc(SB), buf = dalloc(SB), after = dalloc(SB), drift = dalloc(8 * (size_t)V);
    CUdeviceptr eps = dalloc(8), md = dalloc(8);
    h2d(eps, &eps_bar, 8);
    const Kli km = kli("ApplyMask");
    const unsigned run_smem = (unsigned)(sizeof(double) * std::max(kr.threads, 32));
    double export_time = 1.0;
    int n = V;
    auto step = [&]() -> double {
        // ColouredNoise::operator()
        {
            CUdeviceptr a0 = noise, a2 = states_noise;
            void* args[] = {&a0, &n, &a2};
            coop_kli("DoRNG", kr, args, 0);
        }
        CF(cufftExecD2Z(pf, (cufftDoubleReal*)noise, (cufftDoubleComplex*)tmp));
        CK(cuCtxSynchronize());
        {
            CUdeviceptr a0 = tmp, a1 = mask;
            void* args[] = {&a0, &a1, &n};
            coop_kli("ApplyMask", km, args, 0);
        }
        CF(cufftExecZ2D(pr, (cufftDoubleComplex*)tmp, (cufftDoubleReal*)noise));
        CK(cuCtxSynchronize());
        // FermionicDrift::getForce
        {
            CUdeviceptr a0 = eta, a1 = states_f;
            void* args[] = {&a0, &a1, &svol};
            coop("fillNormalRND", args);
            CUdeviceptr z0 = after;
            void* zargs[] = {&z0, &svol};
            coop("setZero_kernel", zargs);
        }
        cg_solve_occupancy(eta, buf, 1, phi, T, B);
        applyD(buf, after, 0, phi, T);
        {
            CUdeviceptr a0 = after, a1 = eta, a2 = drift;
            void* args[] = {&a0, &a1, &a2};
            coop("computeDrift", args);
        }
        // Run and the host copy of eps
        {
            CUdeviceptr a0 = eps, a2 = phi, a3 = drift, a4 = noise, a6 = T.I, a7 = T.J, a8 = T.vals, a9 = md;
            void* args[] = {&a0, &export_time, &a2, &a3, &a4, &n, &a6, &a7, &a8, &a9};
            coop_kli("Run", kr, args, run_smem);
        }
        double h_eps = 0.0;
        CK(cuMemcpyDtoH(&h_eps, eps, 8));
        return h_eps;
    };
    for (int i = 0; i < 3; ++i) step();
    const double t0 = now_s();
    for (int i = 0; i < steps; ++i) step();
    const double t1 = now_s();
    cufftDestroy(pf);
    cufftDestroy(pr);
    FILE* f = std::fopen(out_path, "w");
    if (!f) return 4;
    std::fprintf(f,
                 "{\"lattice\": [%d, %d], \"dirac_ms\": %.6f, \"dirac_gbs_136B\": %.2f, \"cg_solve_ms\": %.6f, "
                 "\"steps\": %d, \"step_ms\": %.6f, \"steps_per_s\": %.4f, \"run_grid\": [%d, %d]}\n",
                 Nt, Nx, ms_dirac, 136.0 * V / (ms_dirac * 1e-3) / 1e9, ms_cg, steps, (t1 - t0) / steps * 1e3,
                 steps / (t1 - t0), kr.blocks, kr.threads);
    std::fclose(f);
    std::printf("ref_harness timing %dx%d ok\n", Nt, Nx);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc < 6) {
        std::fprintf(stderr,
                     "usage: %s fatbin symbols Nt Nx out.bin\n"
                     "       %s fatbin symbols Nt Nx --time field.raw b.raw steps out.json\n",
                     argv[0], argv[0]);
        return 1;
    }
    Nt = std::atoi(argv[3]);
    Nx = std::atoi(argv[4]);
    V = Nt * Nx;
    CK(cuInit(0));
    CUdevice dev;
    CK(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    CK(cuModuleLoad(&mod, argv[1]));
    {
        std::ifstream sf(argv[2]);
        std::string k, m;
        while (sf >> k >> m) {
            CUfunction f;
            CK(cuModuleGetFunction(&f, mod, m.c_str()));
            fns[k] = f;
        }
    }
    if (std::string(argv[5]) == "--time") {
        if (argc < 10) return 1;
        return time_mode(argv[6], argv[7], std::atoi(argv[8]), argv[9]);
    }
    dump = std::fopen(argv[5], "wb");
    if (!dump) return 4;
    put("shape", {(double)Nt, (double)Nx});
    const double m2 = -0.5, lam = 1.0, g = 0.5, m0 = 0.1, eps_bar = 0.02;
    put("params", {m2, lam, g, m0, eps_bar});
    const Tables T = make_tables();
    CGBufs B = make_cg();
    const size_t SB = 64 * (size_t)V;   // bytes of a spinor
    CUdeviceptr M = dalloc(8 * (size_t)V), psi = dalloc(SB), out = dalloc(SB);

    // ---- Dirac operator (r = 1 and r = 0.5)
    std::vector<double> sigma(V), ps(8 * V);
    for (auto& v : sigma) v = unif();
    for (auto& v : ps) v = unif();
    put("sigma", sigma);
    put("psi", ps);
    h2d(M, sigma.data(), 8 * (size_t)V);
    h2d(psi, ps.data(), SB);
    for (double r : {1.0, 0.5}) {
        set_params(m2, lam, g, m0, r, 1.0, 0, eps_bar);
        applyD(psi, out, 0, M, T);
        put(r == 1.0 ? "dirac_D" : "dirac_D_r05", d2h(out, 8 * V));
        applyD(psi, out, 1, M, T);
        put(r == 1.0 ? "dirac_Ddag" : "dirac_Ddag_r05", d2h(out, 8 * V));
    }
    set_params(m2, lam, g, m0, 1.0, 1.0, 0, eps_bar);

    // ---- CG on D^dag D (Dagger) and D D^dag (Normal), reference tolerance
    std::vector<double> b(8 * V);
    for (auto& v : b) v = gauss();
    put("cg_b", b);
    h2d(psi, b.data(), SB);
    cg_solve(psi, out, 1, M, T, B);
    put("cg_x_dag", d2h(out, 8 * V));
    put("cg_rr_dag", d2h(B.rmodsq, 1));
    cg_solve(psi, out, 0, M, T, B);
    put("cg_x_nor", d2h(out, 8 * V));
    put("cg_rr_nor", d2h(B.rmodsq, 1));
    // record of the race: the reference's own launch geometry
    cg_solve_occupancy(psi, out, 1, M, T, B);
    put("cg_x_dag_occupancy", d2h(out, 8 * V));
    put("cg_rr_dag_occupancy", d2h(B.rmodsq, 1));

    // ---- fermion force with injected real eta, normal and rescaled drift mode
    std::vector<double> eta(8 * V, 0.0);
    for (int i = 0; i < 4 * V; ++i) eta[2 * i] = gauss();
    put("force_eta", eta);
    CUdeviceptr deta = dalloc(SB);
    h2d(deta, eta.data(), SB);
    put("force_F", force(deta, M, T, B));
    set_params(m2, lam, g, m0, 1.0, 0.5, 1, eps_bar);
    put("force_F_resc", force(deta, M, T, B));
    set_params(m2, lam, g, m0, 1.0, 1.0, 0, eps_bar);

    // ---- coloured noise (cuFFT D2Z -> ApplyMask -> Z2D)
    std::vector<double> w(V);
    for (auto& v : w) v = gauss();
    put("noise_w", w);
    const double cuts[3] = {0.35355339059327373, 0.25, 1.0};
    for (int i = 0; i < 3; ++i) {
        put(("noise_mask" + std::to_string(i)).c_str(), mask_half(cuts[i]));
        put(("noise_xi" + std::to_string(i)).c_str(), coloured(w, cuts[i]));
    }
    put("noise_cuts", {cuts[0], cuts[1], cuts[2]});

    // ---- Run kernel: bosonic drift, adaptive eps, Euler update
    std::vector<double> phi(V), drift(V), noise(V);
    for (auto& v : phi) v = unif();
    for (auto& v : drift) v = 0.5 * gauss();
    for (auto& v : noise) v = gauss();
    put("run_phi0", phi);
    put("run_force", drift);
    put("run_noise", noise);
    CUdeviceptr dphi = dalloc(8 * (size_t)V), ddr = dalloc(8 * (size_t)V), dno = dalloc(8 * (size_t)V);
    h2d(dphi, phi.data(), 8 * (size_t)V);
    h2d(ddr, drift.data(), 8 * (size_t)V);
    h2d(dno, noise.data(), 8 * (size_t)V);
    double md = 0.0;
    const double e = run_update(dphi, ddr, dno, T, eps_bar, &md);
    put("run_phi1", d2h(dphi, V));
    put("run_drift", d2h(ddr, V));
    put("run_eps", {e, md});

    // ---- observables of the updated field
    {
        const Kli gr = kli("Run");
        const unsigned sm = (unsigned)(sizeof(double) * std::max(gr.threads, 32));
        CUdeviceptr res = dalloc(8 * (size_t)Nt);
        int n = V;
        CUdeviceptr a0 = dphi, a1 = res;
        void* args[] = {&a0, &a1, &n};
        coop_kli("gpuMagnetisation", gr, args, sm);
        put("obs_mag", d2h(res, 1));
        coop_kli("gpuTimeSlices", kli("gpuTimeSlices"), args, sm);
        put("obs_slices", d2h(res, Nt));
        CUdeviceptr s0 = psi, s1 = res;
        h2d(psi, ps.data(), SB);
        int nt = Nt;
        void* a2[] = {&s0, &s1, &nt};
        coop("gpuTimeSlices_spinors", a2);
        put("obs_corr", d2h(res, Nt));
        CUdeviceptr tr = dalloc(8);
        CUdeviceptr f0 = ddr, f1 = tr;
        int vol = V;
        void* a3[] = {&f0, &f1, &vol};
        coop("gpuTraces", a3, 0, 32 * 8);
        put("obs_trace", d2h(tr, 1));
    }

    // ---- three full Langevin steps with injected w and eta (main.cu:370-381)
    {
        const double cut = cuts[0];
        std::vector<double> f(V);
        for (auto& v : f) v = unif();
        put("step_phi0", f);
        h2d(dphi, f.data(), 8 * (size_t)V);
        for (int s = 0; s < 3; ++s) {
            std::vector<double> ws(V), es(8 * V, 0.0);
            for (auto& v : ws) v = gauss();
            for (int i = 0; i < 4 * V; ++i) es[2 * i] = gauss();
            put(("step_w" + std::to_string(s)).c_str(), ws);
            put(("step_eta" + std::to_string(s)).c_str(), es);
            const std::vector<double> xi = coloured(ws, cut);
            h2d(dno, xi.data(), 8 * (size_t)V);
            h2d(deta, es.data(), SB);
            // sigma of D is the current field
            const std::vector<double> cur = d2h(dphi, V);
            h2d(M, cur.data(), 8 * (size_t)V);
            const std::vector<double> F = force(deta, M, T, B);
            h2d(ddr, F.data(), 8 * (size_t)V);
            double mdd = 0.0;
            const double es2 = run_update(dphi, ddr, dno, T, eps_bar, &mdd);
            put(("step_phi" + std::to_string(s + 1)).c_str(), d2h(dphi, V));
            put(("step_eps" + std::to_string(s)).c_str(), {es2, mdd});
        }
        put("step_cut", {cut});
    }
    std::fclose(dump);
    std::printf("ref_harness %dx%d ok\n", Nt, Nx);
    return 0;
}
