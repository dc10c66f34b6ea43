// host_math.hpp -- host-side modular arithmetic and NTT for parameter setup and
// key generation. Exact mod-Q arithmetic, so every routine gives the canonical
// value the reference's '%'-based code gives (nbt.cpp:28-491).
#pragma once
#include <cstdint>
#include <vector>
#include "fheacc.h"

namespace fheacc {
namespace host {

typedef unsigned __int128 u128;

inline uint64_t mulmod(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)((u128)a * b % m); }
inline uint64_t addmod(uint64_t a, uint64_t b, uint64_t m) { uint64_t s = a + b; return s >= m ? s - m : s; }
inline uint64_t submod(uint64_t a, uint64_t b, uint64_t m) { return a >= b ? a - b : a + m - b; }
uint64_t powmod(uint64_t b, uint64_t e, uint64_t m);
bool is_prime(uint64_t x);
uint64_t reverse_bits(uint64_t x, int bits);

// Twiddle tables of one parameter set, in the reference's order
// (params.cpp:149-175): rou[k] = psi^bitrev(k), irou[k] = psi^-bitrev(k).
// Shoup companions w' = floor(w * 2^64 / Q) for the host NTT.
struct Tables {
    int N = 0, logN = 0;
    uint64_t Q = 0, iN = 0;
    std::vector<uint64_t> rou, irou, rou_s, irou_s;
    uint64_t iN_s = 0;
    void build(const fheacc_params &p);
    void ntt(uint64_t *a) const;    // nbt.cpp:423-454, canonical in/out
    void intt(uint64_t *a) const;   // nbt.cpp:456-491, canonical in/out
};

// Validate a parameter set after fheacc_params_derive; returns an error text
// or nullptr.
const char *check_params(const fheacc_params &p);

}  // namespace host
}  // namespace fheacc
