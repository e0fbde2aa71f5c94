// yk_host.h -- host-side helpers of the runtime (no CUDA).
#pragma once

#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "yukawa.h"

namespace yk {

// Minimal TOML reader for the reference's input.toml (sections, key = value,
// strings, booleans, numbers, # comments).  Keys are "section.key".
bool parse_toml(const std::string& path, std::map<std::string, std::string>& kv, std::string& err);

// The cutoff of code/src/colouredNoise.cpp:16-29, 138-145 on the full
// Nt x Nx spectrum: keep[kt*Nx + kx] = 1 if p^2 <= (sqrt(2) pi s)^2, with the
// reference's operation order (boundary modes decide identically).
void momentum_keep(int Nt, int Nx, double cut_fraction, std::vector<uint8_t>& keep);
bool all_modes_kept(int Nt, int Nx, double cut_fraction);

// tw[k] = exp(-2 pi i k / N), k < N, interleaved (re, im).
void twiddles(int N, std::vector<double>& tw);

// POSIX drand48 sequence from glibc's unseeded state, as 1 - 2*drand48()
// (code/src/main.cu:92-95); `skip` values are drawn first.
void drand48_field(int64_t skip, int64_t n, double* out);

// 1 - 2u with u from Philox4x32-10 stream kind 0 of (seed, chain), two values
// per counter (the framework's seeded initial field).
// word3: the counter's last word (0 for sigma, a for pion field a)
void philox_uniform_field(uint64_t seed, uint32_t chain, int64_t n, double* out, uint32_t word3 = 0);

void gamma_method(const double* data, int64_t n, double stau, double out[5]);
// The automatic window of gamma_method from a given Gamma(t), t = 0..tmax, of
// n measurements: fills out[1..4] (error, its error, tau_int, its error).
void gamma_window(const double* gam, int64_t tmax, int64_t n, double stau, double out[5]);

void set_error(const char* fmt, ...);

}  // namespace yk
