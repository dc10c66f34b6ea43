/* A plain C99 client of libfheacc.so (include/fheacc.h), as a runtime written in C
 * would bind it: parameters, seeded keys, LWE encryption and decryption, the
 * on-disk container, context creation (FHEACC_ENODEV without a GPU) and, with a
 * GPU, four gate bootstraps through the blocking host-buffer call, decrypted.
 * Prints "ok <create rc>" and exits 0 when every check holds. */
#include "fheacc.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define CHECK(x)                                                   \
    do {                                                           \
        int rc_ = (x);                                             \
        if (rc_ != FHEACC_OK) {                                    \
            fprintf(stderr, "%s failed: %d\n", #x, rc_);           \
            return 1;                                              \
        }                                                          \
    } while (0)

int main(int argc, char **argv)
{
    const char *path = argc > 1 ? argv[1] : "abi_client.fheacc";
    fheacc_params p;
    CHECK(fheacc_params_preset(0, &p));
    if (p.N != 1024 || p.Q != 134215681ULL) return 2;
    p.n = 32;
    CHECK(fheacc_params_derive(&p));
    uint64_t *sk = malloc((size_t)p.n * sizeof(uint64_t));
    CHECK(fheacc_keygen_lwe_sk(&p, 11, sk));
    const uint8_t bits[4] = {1, 0, 1, 1};
    const size_t w = (size_t)p.n + 1;
    uint64_t *ct = malloc(4 * w * sizeof(uint64_t)), *back = malloc(4 * w * sizeof(uint64_t));
    uint8_t dec[4];
    CHECK(fheacc_lwe_encrypt(&p, 5, sk, bits, 4, ct));
    CHECK(fheacc_lwe_decrypt(&p, sk, ct, 4, dec));
    if (memcmp(dec, bits, 4) != 0) return 3;
    CHECK(fheacc_container_save(path, FHEACC_KIND_LWE_CT, &p, ct, 4 * w));
    CHECK(fheacc_container_load(path, FHEACC_KIND_LWE_CT, &p, back, 4 * w));
    if (memcmp(back, ct, 4 * w * sizeof(uint64_t)) != 0) return 4;
    if (fheacc_container_load(path, FHEACC_KIND_BOOTSTRAP_KEY, &p, back, 4 * w) != FHEACC_EINVAL) return 5;
    fheacc_ctx *ctx = NULL;
    const int rc = fheacc_create(&p, 0, &ctx);
    if (rc == FHEACC_OK) {
        if (fheacc_device_bytes(ctx) == 0) return 6;
        /* NAND, XOR, AND, OR of (1, 1), (0, 1), (1, 1), (0, 1) */
        uint64_t *rsk = malloc((size_t)p.N * sizeof(uint64_t));
        uint64_t *bt = malloc(fheacc_bootstrap_key_words(&p) * sizeof(uint64_t));
        uint64_t *ks = malloc(fheacc_lwe_ks_key_words(&p) * sizeof(uint64_t));
        uint64_t *in = malloc(8 * w * sizeof(uint64_t)), *out = malloc(4 * w * sizeof(uint64_t));
        if (!rsk || !bt || !ks || !in || !out) return 8;
        const uint8_t xy[8] = {1, 0, 1, 0, 1, 1, 1, 1};
        const int32_t gates[4] = {FHEACC_NAND, FHEACC_XOR, FHEACC_AND, FHEACC_OR};
        const uint8_t want[4] = {0, 1, 1, 1};
        CHECK(fheacc_keygen_rlwe_sk(&p, 12, rsk));
        CHECK(fheacc_keygen_bootstrap_key(&p, 13, sk, rsk, bt, 0));
        CHECK(fheacc_keygen_lwe_ks_key(&p, 14, rsk, sk, ks, 0));
        CHECK(fheacc_lwe_encrypt(&p, 6, sk, xy, 8, in));
        CHECK(fheacc_upload_bootstrap_key(ctx, bt, fheacc_bootstrap_key_words(&p)));
        CHECK(fheacc_upload_lwe_ks_key(ctx, ks, fheacc_lwe_ks_key_words(&p)));
        CHECK(fheacc_bootstrap(ctx, in, in + 4 * w, gates, 4, out, 0));
        CHECK(fheacc_lwe_decrypt(&p, sk, out, 4, dec));
        if (memcmp(dec, want, 4) != 0) return 9;
        free(rsk); free(bt); free(ks); free(in); free(out);
        CHECK(fheacc_destroy(ctx));
    } else if (rc != FHEACC_ENODEV) {
        return 7;
    }
    printf("ok %d\n", rc);
    free(sk);
    free(ct);
    free(back);
    return 0;
}
