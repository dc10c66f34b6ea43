"""The boundary from C and C++: a C99 program linked against libfheacc.so
(tests/c_abi/abi_client.c), and the reference-side binding shown in the
integration notes compiled against the reference runtime's own headers."""
import os
import re
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# the reference runtime's headers, through the link oracle/build_ref.sh leaves
REF_INC = os.path.join(ROOT, "oracle", "_ref", "reference", "FHE_ACC_runtime", "include")


def test_c_client_links_and_runs(F, tmp_path):
    lib_dir = os.path.dirname(F.LIB_PATH)
    exe = str(tmp_path / "abi_client")
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                           os.path.join(HERE, "c_abi", "abi_client.c"), "-L", lib_dir, "-lfheacc",
                           "-Wl,-rpath," + lib_dir, "-o", exe])
    r = subprocess.run([exe, str(tmp_path / "ct.fheacc")], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stderr)
    rc = int(r.stdout.split()[1])
    try:
        import torch
        gpu = torch.cuda.is_available()
    except ImportError:
        gpu = False
    assert rc == (F.OK if gpu else F.ENODEV)


@pytest.mark.skipif(not os.path.isdir(REF_INC), reason="reference headers not mounted")
def test_integration_shim_compiles_against_reference_headers(tmp_path):
    """The GPU:: binding a maintainer adds to FHE_ACC_runtime (the C++ block
    of the integration notes) compiles against the runtime's headers and
    include/fheacc.h."""
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    code = re.search(r"```cpp\n(// FHE_ACC_runtime/src/gpu_backend.cpp.*?)```", text, re.S).group(1)
    src = tmp_path / "gpu_backend.cpp"
    src.write_text(code)
    subprocess.check_call(["g++", "-std=c++14", "-fsyntax-only", "-I", REF_INC, "-I", os.path.join(ROOT, "include"),
                           str(src)])
