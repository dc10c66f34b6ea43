// Stand-in for FHE_ACC_runtime/include/LWE.h (see params.h here): the LWE
// ciphertext and key-switch key classes with the runtime's member names and
// layouts (LWE.h:36-101). Test infrastructure.
#pragma once
#include <vector>
#include "params.h"

namespace LWE {
class LWE_ciphertext {
public:
    std::vector<ciphertext_t> a = std::vector<ciphertext_t>(n, 0);
    ciphertext_t b = 0;
};
class keyswitch_key {
public:
    std::vector<std::vector<std::vector<LWE_ciphertext>>> kskey;   // [Bks][digitKS][N]
};
}  // namespace LWE
