// Stand-in for FHE_ACC_runtime/include/app.h (see params.h here): the
// substitution key class (app.h:22-35). Test infrastructure.
#pragma once
#include <vector>
#include "RLWE.h"

namespace application {
class substitute_key {
public:
    std::vector<RLWE::keyswitch_key> subs_key;   // [digitN]
};
}  // namespace application
