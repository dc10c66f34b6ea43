// Stand-in for FHE_ACC_runtime/include/params.h, for building the GPU backend
// (3rd_gen_fhe_acc_gb300/integration/gpu_backend.cpp) where the reference
// runtime is not present. It declares only what the backend reads: the
// runtime's global parameters (params.h:11-110) and enum GATES, with the
// runtime's names and types, so the backend compiles unchanged against
// either header set. Test infrastructure.
#pragma once
#include <cstdint>

typedef uint64_t ciphertext_t;   // nbt.h:26

extern int n;
extern ciphertext_t q;
extern int N;
extern uint16_t digitN;
extern ciphertext_t E_rlwe;
extern ciphertext_t Q;
extern ciphertext_t iN;
extern ciphertext_t ROU;
extern ciphertext_t BGbits;
extern ciphertext_t digitG;
extern ciphertext_t Br;
extern ciphertext_t digitR;
extern ciphertext_t Bks;
extern ciphertext_t digitKS;
extern ciphertext_t Bks_R_bits;
extern ciphertext_t digitKS_R;
enum GATES { OR, AND, NOR, NAND, XOR, XNOR };
extern ciphertext_t gate_constant[6];
