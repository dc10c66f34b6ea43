// Stand-in for FHE_ACC_runtime/include/RLWE.h (see params.h here): the RLWE,
// RGSW, RLWE key-switch and bootstrap key classes with the runtime's member
// names and layouts (RLWE.h:127-345). Test infrastructure.
#pragma once
#include <vector>
#include "params.h"

namespace RLWE {
class RLWE_ciphertext {
public:
    std::vector<ciphertext_t> a = std::vector<ciphertext_t>(N, 0);
    std::vector<ciphertext_t> b = std::vector<ciphertext_t>(N, 0);
    bool NTT_form = true;
};
class keyswitch_key {
public:
    std::vector<RLWE_ciphertext> RLWE_kskey;   // [digitKS_R]
};
class RGSW_ciphertext {
public:
    std::vector<std::vector<RLWE_ciphertext>> c_text;   // [digitG][2]
};
class bootstrap_key {
public:
    std::vector<std::vector<std::vector<RGSW_ciphertext>>> btkey;   // [Br][digitR][n]
};
}  // namespace RLWE
