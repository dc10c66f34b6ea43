// gpu_backend.h -- namespace GPU: the FHE_ACC_runtime's device backend calls
// with the FPGA backend's exact signatures (FHE_ACC_runtime/include/myfpga.h:
// 128-404), implemented over the C ABI of libfheacc.so (include/fheacc.h).
//
// A maintainer adds gpu_backend.cpp to the runtime in place of myfpga.cpp,
// includes this header instead of myfpga.h, and calls GPU:: where the code
// called FPGA::. The slot id becomes a CUDA device index; the PCIe BAR handle
// and the DMA file descriptors are accepted and ignored. Link with -lfheacc
// -lcudart (the expand calls stage through device buffers).
//
// Results: bit-exact with RLWE::eval_bootstrap (RLWE.cpp:726-786), the CPU
// path, which skips residue-0 steps. set_issue_flags(FHEACC_FLAG_FPGA_X1) or
// (FHEACC_FLAG_FPGA_COMPAT) reproduces the FPGA calls' issue orders instead
// (myfpga.cpp:1037-1046 for x1, 1200-1210 for x4..x16).
#ifndef FHEACC_GPU_BACKEND_H
#define FHEACC_GPU_BACKEND_H
#include <cstdint>
#include <memory>
#include <vector>

#include "LWE.h"
#include "RLWE.h"
#include "app.h"
#include "params.h"
#include "fheacc.h"

// The AWS SDK's handle type (fpga_pci.h); a repeated identical typedef is
// harmless where the SDK header is also included.
typedef int pci_bar_handle_t;

namespace GPU {

// 0 if `slot_id` names a CUDA device this backend can use, 1 otherwise
// (check_slot_config, myfpga.cpp:8-62, checks the FPGA image of the slot).
int check_slot_config(int slot_id);
// Number of differing bytes of two buffers (buffer_compare, myfpga.cpp:68-80).
uint64_t buffer_compare(uint8_t *bufa, uint8_t *bufb, size_t buffer_size);

// Creates the device context of `slot_id` (a CUDA device index) from the
// runtime's global parameters (params.h). Replaces OCL_config_wr_rd
// (myfpga.cpp:82-326). 0 on success, -1 on failure.
int OCL_config_wr_rd(const int slot_id);
// The twiddle tables are built when the context is created: these return 0
// (BAR1_ROU_table_{2k,1k}_wr, myfpga.cpp:399-594).
int BAR1_ROU_table_2k_wr(const int slot_id);
int BAR1_ROU_table_1k_wr(const int slot_id);
// Key uploads (dma_write_bootstrap_key, dma_write_subs_key,
// dma_write_RGSW_enc_sk; myfpga.cpp:596-770). 0 on success, -1 on failure.
int dma_write_bootstrap_key(const int slot_id, const RLWE::bootstrap_key &bt_key);
int dma_write_subs_key(const int slot_id, const application::substitute_key &subs_key);
int dma_write_RGSW_enc_sk(const int slot_id, const RLWE::RGSW_ciphertext &enc_sec);
// Read-back verifiers (dma_read_compare_bootstrap_key, _subs_key,
// _RGSW_enc_sk; myfpga.cpp:772-1000): 0 if the slot's device copy is what
// uploading the given key makes (fheacc_verify_bootstrap_key,
// fheacc_verify_subs_key), -1 if it differs or was never uploaded.
int dma_read_compare_bootstrap_key(const int slot_id, const RLWE::bootstrap_key &bt_key);
int dma_read_compare_subs_key(const int slot_id, const application::substitute_key &subs_key);
int dma_read_compare_RGSW_enc_sk(const int slot_id, const RLWE::RGSW_ciphertext &enc_sec);

// Gate bootstrapping (myfpga.cpp:1003-1660). The FPGA runtime key-switches
// on the host and passes the key each call; here the key switch runs on the
// device: the key is uploaded at its first use on a slot, and again whenever
// a different keyswitch_key object is passed. Widths are checked as the
// FPGA calls check them (x4: 4, x8: 8, x12: 12, x16: exactly 10); a width
// mismatch or c1 == c2 gives *rc = -1, a failed allocation -ENOMEM.
LWE::LWE_ciphertext fpga_eval_bootstrap_x1(const LWE::LWE_ciphertext &c1, const LWE::LWE_ciphertext &c2,
                                           const LWE::keyswitch_key &kskey, const GATES gate,
                                           const pci_bar_handle_t ocl_bar_handle, int *rc, int read_fd);
std::vector<LWE::LWE_ciphertext> fpga_eval_bootstrap_x4(const std::vector<LWE::LWE_ciphertext> &c1,
                                                        const std::vector<LWE::LWE_ciphertext> &c2,
                                                        const LWE::keyswitch_key &kskey,
                                                        const std::vector<GATES> gate,
                                                        const pci_bar_handle_t ocl_bar_handle, int *rc, int read_fd);
std::vector<LWE::LWE_ciphertext> fpga_eval_bootstrap_x8(const std::vector<LWE::LWE_ciphertext> &c1,
                                                        const std::vector<LWE::LWE_ciphertext> &c2,
                                                        const LWE::keyswitch_key &kskey,
                                                        const std::vector<GATES> gate,
                                                        const pci_bar_handle_t ocl_bar_handle, int *rc, int read_fd);
std::vector<LWE::LWE_ciphertext> fpga_eval_bootstrap_x12(const std::vector<LWE::LWE_ciphertext> &c1,
                                                         const std::vector<LWE::LWE_ciphertext> &c2,
                                                         const LWE::keyswitch_key &kskey,
                                                         const std::vector<GATES> gate,
                                                         const pci_bar_handle_t ocl_bar_handle, int *rc, int read_fd);
std::vector<LWE::LWE_ciphertext> fpga_eval_bootstrap_x16(const std::vector<LWE::LWE_ciphertext> &c1,
                                                         const std::vector<LWE::LWE_ciphertext> &c2,
                                                         const LWE::keyswitch_key &kskey,
                                                         const std::vector<GATES> gate,
                                                         const pci_bar_handle_t ocl_bar_handle, int *rc, int read_fd);

// RLWE::eval_bootstrap (RLWE.cpp:726-786) with its own signature, for code
// that called the CPU path: on the lowest configured slot, uploading btkey
// the first time this key object is passed (and again when another one is)
// and the key switch key as the calls above do. c1 == c2, which the CPU path
// answers with exit(1), and device errors return a default-constructed
// (all-zero) ciphertext, as the FPGA calls do.
LWE::LWE_ciphertext eval_bootstrap(const LWE::LWE_ciphertext &c1, const LWE::LWE_ciphertext &c2,
                                   const RLWE::bootstrap_key &btkey, const LWE::keyswitch_key &kskey, const GATES gate);

// expand_RLWE on the device (myfpga.cpp:1662-1790): N RLWEs, result[i] =
// RLWE(N b_i X^i) for the input RLWE(sum b_i X^i) in the NTT domain. Needs
// dma_write_subs_key. NULL and *rc != 0 on failure.
std::unique_ptr<std::vector<RLWE::RLWE_ciphertext>> fpga_expand_RLWE(const RLWE::RLWE_ciphertext &c1,
                                                                     const pci_bar_handle_t ocl_bar_handle, int *rc,
                                                                     int read_fd, int write_fd);
// The reference's two DMA-issue variants of expand_RLWE (continuous and
// batched reads and writes, myfpga.cpp:1797-1956 and 1959-2275) compute the
// same N RLWEs; here they are the same device call.
std::unique_ptr<std::vector<RLWE::RLWE_ciphertext>> fpga_expand_RLWE_cont_rd_wr(const RLWE::RLWE_ciphertext &c1,
                                                                                const pci_bar_handle_t ocl_bar_handle,
                                                                                int *rc, int read_fd, int write_fd);
std::unique_ptr<std::vector<RLWE::RLWE_ciphertext>> fpga_expand_RLWE_batch_rd_wr(const RLWE::RLWE_ciphertext &c1,
                                                                                 const pci_bar_handle_t ocl_bar_handle,
                                                                                 int *rc, int read_fd, int write_fd);
// homo_expand on the device (myfpga.cpp:2278-2452): digitG packed RLWEs to N
// RGSWs. Needs dma_write_subs_key and dma_write_RGSW_enc_sk.
std::shared_ptr<std::vector<RLWE::RGSW_ciphertext>> fpga_homo_expand(
    const std::unique_ptr<std::vector<RLWE::RLWE_ciphertext>> &packed_bits, const pci_bar_handle_t ocl_bar_handle,
    int *rc, int read_fd, int write_fd);

// The PSI operations the reference runs on the CPU (RLWE::CMUX and
// RLWE::blind_rotate, RLWE.cpp:788-793 and 824-838), with their signatures,
// on the lowest configured slot: CMUX of NTT-domain RLWEs; blind_rotate with
// log2 N RGSWs (num_rotate_poly, params.h), its input moved to the NTT domain
// first as the CPU path does. An error returns a default-constructed
// ciphertext where the CPU path would exit(1).
RLWE::RLWE_ciphertext CMUX(const RLWE::RLWE_ciphertext &c0, const RLWE::RLWE_ciphertext &c1,
                           const RLWE::RGSW_ciphertext &SEL);
RLWE::RLWE_ciphertext blind_rotate(const RLWE::RLWE_ciphertext &c_in, const bool forward,
                                   const std::vector<RLWE::RGSW_ciphertext> &C);

// Not in the FPGA API: the issue order of the bootstrap calls (0, the
// default: the CPU path's; FHEACC_FLAG_FPGA_X1 or FHEACC_FLAG_FPGA_COMPAT),
// the context of a slot for direct use of the C ABI, and its release.
void set_issue_flags(uint32_t flags);
fheacc_ctx *context(const int slot_id);
int release(const int slot_id);

}  // namespace GPU

#endif
