// container.cpp -- the on-disk container for keys and ciphertexts.
//
// The reference keeps keys and ciphertexts only in process memory (std::vector
// value objects) and regenerates them every run from std::random_device
// (RNG.cpp:3-37). This file gives the library one self-describing binary
// format so that generated key sets, encrypted inputs and results can be
// written once and read by any later process on either machine:
//
//   offset  size  field
//   0       8     magic "FHEACC01"
//   8       4     kind (FHEACC_KIND_*)
//   12      4     header bytes (64)
//   16      8     fingerprint of the parameter set (FNV-1a of its fields)
//   24      8     number of 64-bit words that follow the header
//   32      8     FNV-1a 64 of the words
//   40      24    reserved (zero)
//   64      ...   the words, little endian, in the library's host layouts
//
// A load checks the magic, the kind, the parameter fingerprint, the size the
// caller expects and the checksum, and fails with an error code otherwise.
#include "fheacc.h"
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

constexpr char kMagic[8] = {'F', 'H', 'E', 'A', 'C', 'C', '0', '1'};
constexpr uint32_t kHeader = 64;

uint64_t fnv1a(uint64_t h, const void *p, size_t n)
{
    const unsigned char *b = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < n; i++) {
        h ^= b[i];
        h *= 0x100000001B3ULL;
    }
    return h;
}

uint64_t params_fingerprint(const fheacc_params &p)
{
    const uint64_t f[] = {(uint64_t)p.n, p.q, (uint64_t)p.N, p.Q, p.BG_bits, p.digitG, p.Br, p.digitR,
                          p.Bks, p.digitKS, p.Bks_R_bits, p.digitKS_R, p.gate_constant[0], p.gate_constant[1],
                          p.gate_constant[2], p.gate_constant[3], p.gate_constant[4], p.gate_constant[5]};
    return fnv1a(0xCBF29CE484222325ULL, f, sizeof f);
}

void put64(unsigned char *d, uint64_t v)
{
    for (int i = 0; i < 8; i++) d[i] = (unsigned char)(v >> (8 * i));
}

uint64_t get64(const unsigned char *d)
{
    uint64_t v = 0;
    for (int i = 0; i < 8; i++) v |= (uint64_t)d[i] << (8 * i);
    return v;
}

}  // namespace

extern "C" int fheacc_container_save(const char *path, uint32_t kind, const fheacc_params *p,
                                     const uint64_t *words, size_t count)
{
    if (!path || !p || (count && !words)) return FHEACC_EINVAL;
    unsigned char h[kHeader] = {};
    std::memcpy(h, kMagic, 8);
    for (int i = 0; i < 4; i++) h[8 + i] = (unsigned char)(kind >> (8 * i));
    for (int i = 0; i < 4; i++) h[12 + i] = (unsigned char)(kHeader >> (8 * i));
    put64(h + 16, params_fingerprint(*p));
    put64(h + 24, count);
    uint64_t sum = 0xCBF29CE484222325ULL;
    std::vector<unsigned char> buf;
    FILE *f = std::fopen(path, "wb");
    if (!f) return FHEACC_EIO;
    // checksum over the little-endian bytes, written in chunks
    const size_t chunk = 1 << 16;
    buf.resize(chunk * 8);
    bool ok = std::fwrite(h, 1, kHeader, f) == kHeader;
    for (size_t at = 0; ok && at < count; at += chunk) {
        const size_t n = count - at < chunk ? count - at : chunk;
        for (size_t i = 0; i < n; i++) put64(buf.data() + 8 * i, words[at + i]);
        sum = fnv1a(sum, buf.data(), 8 * n);
        ok = std::fwrite(buf.data(), 1, 8 * n, f) == 8 * n;
    }
    put64(h + 32, sum);
    ok = ok && std::fseek(f, 0, SEEK_SET) == 0 && std::fwrite(h, 1, kHeader, f) == kHeader;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? FHEACC_OK : FHEACC_EIO;
}

extern "C" int fheacc_container_info(const char *path, uint32_t *kind, uint64_t *fingerprint, size_t *count)
{
    if (!path) return FHEACC_EINVAL;
    FILE *f = std::fopen(path, "rb");
    if (!f) return FHEACC_EIO;
    unsigned char h[kHeader];
    const bool ok = std::fread(h, 1, kHeader, f) == kHeader && std::memcmp(h, kMagic, 8) == 0;
    std::fclose(f);
    if (!ok) return FHEACC_EINVAL;
    if (kind) *kind = (uint32_t)h[8] | (uint32_t)h[9] << 8 | (uint32_t)h[10] << 16 | (uint32_t)h[11] << 24;
    if (fingerprint) *fingerprint = get64(h + 16);
    if (count) *count = (size_t)get64(h + 24);
    return FHEACC_OK;
}

extern "C" int fheacc_container_load(const char *path, uint32_t kind, const fheacc_params *p, uint64_t *words,
                                     size_t count)
{
    if (!path || !p || (count && !words)) return FHEACC_EINVAL;
    uint32_t k = 0;
    uint64_t fp = 0;
    size_t n = 0;
    int rc = fheacc_container_info(path, &k, &fp, &n);
    if (rc) return rc;
    if (k != kind || fp != params_fingerprint(*p) || n != count) return FHEACC_EINVAL;
    FILE *f = std::fopen(path, "rb");
    if (!f) return FHEACC_EIO;
    unsigned char h[kHeader];
    bool ok = std::fread(h, 1, kHeader, f) == kHeader;
    uint64_t sum = 0xCBF29CE484222325ULL;
    const size_t chunk = 1 << 16;
    std::vector<unsigned char> buf(chunk * 8);
    for (size_t at = 0; ok && at < count; at += chunk) {
        const size_t m = count - at < chunk ? count - at : chunk;
        ok = std::fread(buf.data(), 1, 8 * m, f) == 8 * m;
        if (!ok) break;
        sum = fnv1a(sum, buf.data(), 8 * m);
        for (size_t i = 0; i < m; i++) words[at + i] = get64(buf.data() + 8 * i);
    }
    std::fclose(f);
    if (!ok) return FHEACC_EIO;
    return sum == get64(h + 32) ? FHEACC_OK : FHEACC_EIO;
}
