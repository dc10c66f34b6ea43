"""The boundary from C and C++:
- a C99 program linked against libfheacc.so (tests/c_abi/abi_client.c), which
  on a GPU also bootstraps four gates through the blocking host-buffer call;
- the GPU:: backend a maintainer adds to FHE_ACC_runtime in place of the FPGA
  backend (3rd_gen_fhe_acc_gb300/integration/gpu_backend.cpp, the FPGA::
  signatures of myfpga.h:128-404), compiled against the runtime's own headers
  where the reference is mounted, and built with a C++ client
  (tests/c_abi/shim_client.cpp) against the stand-in headers of
  tests/c_abi/runtime_api; on a GPU the client runs the fixed-width bootstrap
  calls, expand_RLWE and homo_expand through it."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
INTEG = os.path.join(ROOT, "3rd_gen_fhe_acc_gb300", "integration")
# the reference runtime's headers, through the link oracle/build_ref.sh leaves
REF_INC = os.path.join(ROOT, "oracle", "_ref", "reference", "FHE_ACC_runtime", "include")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


def test_c_client_links_and_runs(F, tmp_path):
    lib_dir = os.path.dirname(F.LIB_PATH)
    exe = str(tmp_path / "abi_client")
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                           os.path.join(HERE, "c_abi", "abi_client.c"), "-L", lib_dir, "-lfheacc",
                           "-Wl,-rpath," + lib_dir, "-o", exe])
    r = subprocess.run([exe, str(tmp_path / "ct.fheacc")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    rc = int(r.stdout.split()[1])
    assert rc == (F.OK if _has_gpu() else F.ENODEV)


@pytest.mark.skipif(not os.path.isdir(REF_INC), reason="reference headers not mounted")
def test_gpu_backend_compiles_against_reference_headers():
    """gpu_backend.cpp compiles unchanged against the runtime's params.h,
    LWE.h, RLWE.h and app.h (C++14, the runtime's standard)."""
    subprocess.check_call(["g++", "-std=c++14", "-fsyntax-only", "-Wall", "-Wextra", "-I", REF_INC, "-I", INTEG,
                           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
                           os.path.join(INTEG, "gpu_backend.cpp")])


def _build_shim_client(F, out):
    lib_dir = os.path.dirname(F.LIB_PATH)
    subprocess.check_call(["g++", "-std=c++14", "-O1", "-Wall", "-Wextra", "-Werror",
                           "-I", os.path.join(HERE, "c_abi", "runtime_api"), "-I", INTEG,
                           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
                           os.path.join(HERE, "c_abi", "shim_client.cpp"), os.path.join(INTEG, "gpu_backend.cpp"),
                           "-L", lib_dir, "-lfheacc", "-L", os.path.join(CUDA, "lib64"), "-lcudart",
                           "-Wl,-rpath," + lib_dir, "-Wl,-rpath," + os.path.join(CUDA, "lib64"), "-o", out])


def test_gpu_backend_builds_with_client(F, tmp_path):
    _build_shim_client(F, str(tmp_path / "shim_client"))


@pytest.mark.gpu
def test_gpu_backend_runs_fpga_calls(F, tmp_path):
    """Through GPU::fpga_eval_bootstrap_x4/x8/x12/x16/x1 (4, 8, 12 and exactly
    10 gates; refused sizes and c1 == c2 give rc = -1), fpga_expand_RLWE (and
    its _cont_rd_wr and _batch_rd_wr variants) and fpga_homo_expand: outputs
    decrypt and equal the C ABI's words."""
    exe = str(tmp_path / "shim_client")
    _build_shim_client(F, exe)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, (r.stdout, r.stderr)
    assert "shim ok" in r.stdout
