// yk_host.cpp -- parameter surface and host helpers of the runtime:
// input.toml parsing and the reference's parameter conversion
// (code/src/main.cu:58-63, 112-170), the momentum cutoff
// (code/src/colouredNoise.cpp:16-29, 138-145), FFT twiddles, the reference's
// drand48 initial field and Wolff's Gamma-method.
#include "yk_host.h"

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>

namespace yk {

static thread_local std::string g_error;

void set_error(const char* fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_error = buf;
}

static std::string trim(const std::string& s)
{
    size_t a = 0, b = s.size();
    while (a < b && (s[a] == ' ' || s[a] == '\t' || s[a] == '\r')) ++a;
    while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\t' || s[b - 1] == '\r')) --b;
    return s.substr(a, b - a);
}

bool parse_toml(const std::string& path, std::map<std::string, std::string>& kv, std::string& err)
{
    std::ifstream in(path);
    if (!in) {
        err = "cannot open " + path;
        return false;
    }
    std::string line, section;
    int lineno = 0;
    while (std::getline(in, line)) {
        ++lineno;
        // strip a comment that is not inside a string
        bool instr = false;
        for (size_t i = 0; i < line.size(); ++i) {
            if (line[i] == '"') instr = !instr;
            if (line[i] == '#' && !instr) {
                line.resize(i);
                break;
            }
        }
        line = trim(line);
        if (line.empty()) continue;
        if (line[0] == '[') {
            const size_t e = line.find(']');
            if (e == std::string::npos) {
                err = path + ":" + std::to_string(lineno) + ": bad section header";
                return false;
            }
            section = trim(line.substr(1, e - 1));
            continue;
        }
        const size_t eq = line.find('=');
        if (eq == std::string::npos) {
            err = path + ":" + std::to_string(lineno) + ": expected key = value";
            return false;
        }
        std::string key = trim(line.substr(0, eq));
        std::string val = trim(line.substr(eq + 1));
        if (val.size() >= 2 && val.front() == '"' && val.back() == '"') val = val.substr(1, val.size() - 2);
        kv[section.empty() ? key : section + "." + key] = val;
    }
    return true;
}

// p^2 of mode (kt, kx): (coo <= L/2 ? coo : coo - L) * 2.0 * M_PI / L, summed
// over the two directions in order (colouredNoise.cpp:16-29).
static double momentum_sq(int kt, int kx, int Nt, int Nx)
{
    const int sizes[2] = {Nt, Nx};
    const int coo[2] = {kt, kx};
    double msq = 0.0;
    for (int d = 0; d < 2; ++d) {
        const int L = sizes[d];
        const double tmp = (coo[d] <= (L / 2) ? coo[d] : coo[d] - L) * 2.0 * M_PI / L;
        msq += tmp * tmp;
    }
    return msq;
}

static double cut_sq(double s)
{
    const double c = std::sqrt(2.0) * M_PI * s;   // colouredNoise.cpp:139
    return c * c;
}

void momentum_keep(int Nt, int Nx, double cut_fraction, std::vector<uint8_t>& keep)
{
    const double csq = cut_sq(cut_fraction);
    keep.assign((size_t)Nt * Nx, 0);
    for (int kt = 0; kt < Nt; ++kt)
        for (int kx = 0; kx < Nx; ++kx) {
            // the reference evaluates the half spectrum kx <= Nx/2; the other
            // half is its k -> -k mirror
            const int kxh = (kx <= Nx / 2) ? kx : Nx - kx;
            const int kth = (kx <= Nx / 2) ? kt : (Nt - kt) % Nt;
            keep[(size_t)kt * Nx + kx] = (momentum_sq(kth, kxh, Nt, Nx) <= csq) ? 1 : 0;
        }
}

bool all_modes_kept(int Nt, int Nx, double cut_fraction)
{
    const double csq = cut_sq(cut_fraction);
    for (int kt = 0; kt < Nt; ++kt)
        for (int kx = 0; kx <= Nx / 2; ++kx)
            if (!(momentum_sq(kt, kx, Nt, Nx) <= csq)) return false;
    return true;
}

void twiddles(int N, std::vector<double>& tw)
{
    tw.resize(2 * (size_t)N);
    const long double two_pi = 6.283185307179586476925286766559005768L;
    for (int k = 0; k < N; ++k) {
        const long double a = -two_pi * (long double)k / (long double)N;
        tw[2 * k] = (double)cosl(a);
        tw[2 * k + 1] = (double)sinl(a);
    }
}

void drand48_field(int64_t skip, int64_t n, double* out)
{
    // X <- (0x5DEECE66D X + 0xB) mod 2^48, X0 = 0 (glibc, no seeding call);
    // drand48() = X / 2^48.
    uint64_t X = 0;
    const uint64_t mask = (1ULL << 48) - 1;
    for (int64_t i = 0; i < skip; ++i) X = (0x5DEECE66DULL * X + 0xBULL) & mask;
    for (int64_t i = 0; i < n; ++i) {
        X = (0x5DEECE66DULL * X + 0xBULL) & mask;
        out[i] = 1.0 - 2.0 * ((double)X * 0x1p-48);
    }
}

static void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int round = 0; round < 10; ++round) {
        if (round > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        c[1] = (uint32_t)p1;
        c[3] = (uint32_t)p0;
        c[0] = n0;
        c[2] = n2;
    }
}

static double u52(uint32_t hi, uint32_t lo)
{
    const uint64_t m = ((uint64_t)hi << 20) | (lo >> 12);
    return ((double)m + 0.5) * 0x1p-52;
}

void philox_uniform_field(uint64_t seed, uint32_t chain, int64_t n, double* out, uint32_t word3)
{
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32) ^ chain;
    for (int64_t e = 0; e < (n + 1) / 2; ++e) {
        uint32_t c[4] = {(uint32_t)e, 0u, 0u, word3};
        philox4x32_10(c, k0, k1);
        out[2 * e] = 1.0 - 2.0 * u52(c[0], c[1]);
        if (2 * e + 1 < n) out[2 * e + 1] = 1.0 - 2.0 * u52(c[2], c[3]);
    }
}

// U. Wolff, "Monte Carlo errors with less errors", Comput. Phys. Commun. 156
// (2004) 143: autocorrelation function, automatic window W with S_tau,
// bias-corrected Gamma, error, error of the error, tau_int and its error.
void gamma_method(const double* data, int64_t n, double stau, double out[5])
{
    double mean = 0.0;
    for (int64_t i = 0; i < n; ++i) mean += data[i];
    mean /= (double)(n > 0 ? n : 1);
    out[0] = mean;
    out[1] = out[2] = out[3] = out[4] = 0.0;
    if (n < 2) return;
    const int64_t tmax = n / 2;
    std::vector<double> gam((size_t)tmax + 1);
    for (int64_t t = 0; t <= tmax; ++t) {
        double s = 0.0;
        for (int64_t i = 0; i + t < n; ++i) s += (data[i] - mean) * (data[i + t] - mean);
        gam[(size_t)t] = s / (double)(n - t);
    }
    gamma_window(gam.data(), tmax, n, stau, out);
}

// The automatic window and the errors from Gamma(t), t = 0..tmax, of n
// measurements: fills out[1..4] (error, error of error, tau_int, its error).
void gamma_window(const double* gam_in, int64_t tmax, int64_t n, double stau, double out[5])
{
    out[1] = out[2] = out[3] = out[4] = 0.0;
    if (n < 2 || tmax < 1 || gam_in[0] == 0.0) return;
    std::vector<double> gam(gam_in, gam_in + tmax + 1);
    int64_t W = tmax;
    double gint = 0.0;
    for (int64_t t = 1; t <= tmax; ++t) {
        gint += gam[(size_t)t] / gam[0];
        const double tauw = (gint <= 0.0) ? 1e-5 : stau / std::log((gint + 1.0) / gint);
        const double gw = std::exp(-(double)t / tauw) - tauw / std::sqrt((double)t * (double)n);
        if (gw < 0.0) {
            W = t;
            break;
        }
    }
    double cf = gam[0];
    for (int64_t t = 1; t <= W; ++t) cf += 2.0 * gam[(size_t)t];
    for (auto& g : gam) g += cf / (double)n;
    double cf2 = gam[0], acc = gam[0];
    for (int64_t t = 1; t <= W; ++t) {
        cf2 += 2.0 * gam[(size_t)t];
        acc += gam[(size_t)t];
    }
    const double tau = acc / gam[0] - 0.5;
    out[1] = std::sqrt(cf2 / (double)n);
    out[2] = out[1] * std::sqrt(((double)W + 0.5) / (double)n);
    out[3] = tau;
    out[4] = tau * 2.0 * std::sqrt(((double)W - tau + 0.5) / (double)n);
}

}  // namespace yk

// ---------------------------------------------------------------------------
// C ABI: parameters
// ---------------------------------------------------------------------------
extern "C" {

const char* yk_last_error(void) { return yk::g_error.c_str(); }

const char* yk_version(void) { return "yukawa_gb300 1.0 (sm_103a)"; }

void yk_params_default(yk_params* p)
{
    std::memset(p, 0, sizeof(*p));
    // code/input.toml:1-28
    p->use_mass = 0;
    p->mass = 0.2;
    p->g = 0.0;
    p->kappa = 0.18;
    p->lambda = 0.02;
    p->cut_fraction = 1.0;
    p->average_epsilon = 0.02;
    p->max_langevin_time = 100.0;
    p->export_time = 0.5;
    p->burn_count = 10;
    p->measure_drift_count = 10;
    p->seed = 1234;
    p->yukawa_coupling = 1.0;
    p->fermion_mass = 1.0;
    p->drift_mode = 0;
    p->wilson_param = 1.0;
    // code/src/params.h:13-15, 28
    p->Nt = 16;
    p->Nx = 16;
    p->precision = YK_FP64;
    p->n_rhs = 1;
    p->cg_tol_mode = YK_TOL_ABS;
    p->cg_tol = 1e-8;
    p->cg_max_iter = 1000;
    p->reliable_every = 0;
    p->reliable_delta = 0.001;
    p->fixed_dt = 0.0;
    p->init = YK_INIT_DRAND48;
    p->learned_layers = 0;
}

static bool get_d(const std::map<std::string, std::string>& kv, const char* k, double* v)
{
    auto it = kv.find(k);
    if (it == kv.end()) return false;
    *v = std::strtod(it->second.c_str(), nullptr);
    return true;
}

static bool get_i(const std::map<std::string, std::string>& kv, const char* k, int* v)
{
    auto it = kv.find(k);
    if (it == kv.end()) return false;
    *v = (int)std::strtol(it->second.c_str(), nullptr, 10);
    return true;
}

int yk_params_from_toml(const char* path, yk_params* p)
{
    yk_params_default(p);
    std::map<std::string, std::string> kv;
    std::string err;
    if (!yk::parse_toml(path, kv, err)) {
        yk::set_error("%s", err.c_str());
        return YK_EIO;
    }
    auto s = [&](const char* k) -> std::string {
        auto it = kv.find(k);
        return it == kv.end() ? std::string() : it->second;
    };
    // [physics] (main.cu:114-131)
    if (kv.count("physics.useMass")) p->use_mass = (s("physics.useMass") == "true") ? 1 : 0;
    get_d(kv, "physics.mass", &p->mass);
    get_d(kv, "physics.g", &p->g);
    get_d(kv, "physics.kappa", &p->kappa);
    get_d(kv, "physics.lambda", &p->lambda);
    get_d(kv, "physics.cutFraction", &p->cut_fraction);
    // [langevin] (main.cu:136-141)
    get_d(kv, "langevin.averageEpsilon", &p->average_epsilon);
    get_d(kv, "langevin.MaxLangevinTime", &p->max_langevin_time);
    get_d(kv, "langevin.ExportTime", &p->export_time);
    get_i(kv, "langevin.burnCount", &p->burn_count);
    get_i(kv, "langevin.MeasureDriftCount", &p->measure_drift_count);
    // [random] (main.cu:133-134)
    if (kv.count("random.seed")) p->seed = std::strtoll(s("random.seed").c_str(), nullptr, 10);
    // [fermions] (main.cu:162-170)
    get_d(kv, "fermions.yukawa_coupling", &p->yukawa_coupling);
    get_d(kv, "fermions.fermion_mass", &p->fermion_mass);
    get_i(kv, "fermions.driftMode", &p->drift_mode);
    get_d(kv, "fermions.WilsonParam", &p->wilson_param);
    // [lattice]: the compile-time Sizes of params.h:28, as runs.py:80-85 sets them
    get_i(kv, "lattice.Nt", &p->Nt);
    get_i(kv, "lattice.Nx", &p->Nx);
    // [gpu] extensions
    if (kv.count("gpu.precision")) {
        const std::string v = s("gpu.precision");
        p->precision = (v == "mixed" || v == "2") ? YK_MIXED : YK_FP64;
    }
    get_i(kv, "gpu.n_rhs", &p->n_rhs);
    if (kv.count("gpu.cg_tol_mode")) {
        const std::string v = s("gpu.cg_tol_mode");
        p->cg_tol_mode = (v == "rel" || v == "1") ? YK_TOL_REL : YK_TOL_ABS;
    }
    get_d(kv, "gpu.cg_tol", &p->cg_tol);
    get_i(kv, "gpu.cg_max_iter", &p->cg_max_iter);
    get_i(kv, "gpu.reliable_every", &p->reliable_every);
    get_d(kv, "gpu.reliable_delta", &p->reliable_delta);
    get_d(kv, "gpu.fixed_dt", &p->fixed_dt);
    if (kv.count("gpu.init")) {
        const std::string v = s("gpu.init");
        p->init = (v == "philox") ? YK_INIT_PHILOX : (v == "none" ? YK_INIT_NONE : YK_INIT_DRAND48);
    }
    get_i(kv, "gpu.learned_layers", &p->learned_layers);
    if (kv.count("gpu.pions")) {
        const std::string v = s("gpu.pions");
        p->pions = (v == "true" || v == "1") ? 1 : 0;
    }
    // a network has 2..8 layers (yk_net_setup); refuse other values here,
    // before a run spends its thermalisation on a setting it cannot use
    if (p->learned_layers != 0 && (p->learned_layers < 2 || p->learned_layers > 8)) {
        yk::set_error("yk_params_from_toml: gpu.learned_layers = %d (0 for off, or 2..8)", p->learned_layers);
        return YK_EINVAL;
    }
    return YK_OK;
}

int yk_derive_action(const yk_params* p, yk_action* a)
{
    if (!p || !a) {
        yk::set_error("yk_derive_action: null argument");
        return YK_EINVAL;
    }
    std::memset(a, 0, sizeof(*a));
    const double nd2 = 2.0 * 2.0;   // 2 * nDim, nDim = 2 (params.h:23)
    if (p->use_mass) {
        // main.cu:117-122 and FindKappa main.cu:58-63
        a->m2 = p->mass;
        a->lambda = p->g;
        const double delta = (nd2 + p->mass) * (nd2 + p->mass) + 4.0 * p->g / 3.0;
        a->kappa = (-(nd2 + p->mass) + std::sqrt(delta)) / (2.0 * p->g / 3.0);
    } else {
        // main.cu:123-129
        a->kappa = p->kappa;
        a->m2 = (1.0 - 2.0 * p->lambda) / p->kappa - nd2;
        a->lambda = 6.0 * p->lambda / (p->kappa * p->kappa);
    }
    a->sq2kappa = std::sqrt(2.0 * a->kappa);                                    // main.cu:130
    a->g = p->use_mass ? p->yukawa_coupling : p->yukawa_coupling / a->sq2kappa; // main.cu:166-169
    a->m0 = p->fermion_mass;
    a->r = p->wilson_param;
    a->cut_fraction = p->cut_fraction;
    a->eps_bar = p->average_epsilon;
    a->drift_mode = p->drift_mode;
    a->use_mass = p->use_mass;
    return YK_OK;
}

int yk_gamma_method(const double* data, int64_t n, double stau, double* out5)
{
    if (!data || !out5 || n < 0) {
        yk::set_error("yk_gamma_method: bad arguments");
        return YK_EINVAL;
    }
    yk::gamma_method(data, n, stau, out5);
    return YK_OK;
}

}  // extern "C"
