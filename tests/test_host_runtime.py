"""Host side, no GPU: parameter derivation, the C ABI's exported symbols, seeded
key generation (deterministic across machines), encryption, and the oracle
against outputs of the reference's own eval_bootstrap."""
import ctypes
import hashlib
import json
import os
import re

import numpy as np
import pytest

from conftest import KeySet
from oracle_lib import ROOT

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def header_functions():
    with open(os.path.join(ROOT, "include", "fheacc.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(fheacc_\w+)\s*\(", text)))


def test_abi_exports_every_declared_symbol(F):
    L = ctypes.CDLL(F.LIB_PATH)
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_presets_match_reference_params(F):
    with open(os.path.join(GOLD, "params.json")) as f:
        ref = json.load(f)
    p0 = F.params_preset(0)
    assert (p0.Q, p0.iN, p0.ROU) == (ref["1k"]["Q"], ref["1k"]["iN"], ref["1k"]["ROU"])
    assert (p0.digitG, p0.digitR, p0.digitKS, p0.digitKS_R) == (4, 2, 6, 3)
    assert list(p0.gate_constant) == [320, 448, 64, 192, 320, 64]
    p1 = F.params_preset(1)
    assert (p1.Q, p1.iN, p1.ROU) == (ref["2k"]["Q"], ref["2k"]["iN"], ref["2k"]["ROU"])
    assert (p1.digitG, p1.digitR, p1.digitKS, p1.digitKS_R) == (6, 2, 12, 6)
    p2 = F.params_preset(2)
    assert (p2.n, p2.digitG, p2.BG_bits) == (512, 3, 9)


def test_twiddles_match_oracle(F, keys0):
    rou, irou = F.twiddle_tables(keys0.P)
    orou, oirou = keys0.oracle.tables()
    assert np.array_equal(rou, orou) and np.array_equal(irou, oirou)


def test_invalid_params_rejected(F):
    p = F.params_preset(0)
    p.Q = p.Q + 2          # not prime / not 1 mod 2N
    with pytest.raises(F.FheaccError):
        F.derive(p)
    p = F.params_preset(0)
    p.q = 500              # not a power of two
    with pytest.raises(F.FheaccError):
        F.derive(p)
    for preset in (0, 1):
        p = F.params_preset(preset)
        p.BG_bits, p.digitG = 6, 4  # BG^digitG = 2^24 does not cover Q
        with pytest.raises(F.FheaccError):
            F.derive(p)


def test_context_without_gpu_fails_cleanly(F):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(F.FheaccError) as e:
        F.Context(F.params_preset(0), 0)
    assert e.value.code == F.ENODEV
    # entry points given no context return EINVAL instead of touching memory
    import ctypes
    n = ctypes.c_uint64()
    assert F.lib().fheacc_kernel_launches(None, ctypes.byref(n)) == F.EINVAL


def test_keygen_deterministic_and_distributions(F, keys0):
    P = keys0.P
    again = F.LWE_secretkey(P, 11)
    assert np.array_equal(again, keys0.lwe_sk)
    vals = set(np.unique(keys0.lwe_sk).tolist())
    assert vals <= {0, 1, P.q - 1}
    # RLWE secret: ternary in the time domain
    z = keys0.oracle.intt(keys0.rlwe_sk)
    assert set(np.unique(z).tolist()) <= {0, 1, P.Q - 1}
    # a bootstrap-key RLWE row decrypts to its plaintext plus small noise
    ph = F.RLWE_phase(P, keys0.rlwe_sk, keys0.btkey[:2 * P.N].copy())
    noise = np.minimum(ph, P.Q - ph)
    assert noise.max() < P.Q // 1000 or (noise > P.Q // 1000).sum() == 1


def test_keys_match_reference_fixture_seeds(F, keys0):
    """Keys and ciphertexts regenerate bit-identically from the fixture's
    seeds on this machine (the generator is integer-only)."""
    fx = np.load(os.path.join(GOLD, "ref_bootstrap_p0.npz"))
    h = hashlib.sha256()
    for a in (keys0.lwe_sk, keys0.rlwe_sk, keys0.btkey[:1 << 20], keys0.kskey[:1 << 20]):
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.hexdigest() == fx["keys_sha256"].item().decode()


def test_encrypt_decrypt_roundtrip(F, keys0):
    bits = np.random.default_rng(3).integers(0, 2, 2000).astype(np.uint8)
    ct = keys0.encrypt(bits, seed=5)
    assert np.array_equal(keys0.decrypt(ct), bits)


def test_oracle_equals_reference_outputs(F, keys0):
    """The oracle's eval_bootstrap on the fixture's inputs gives exactly the
    words the reference produced (tests/golden/make_ref_fixtures.py)."""
    import sys
    sys.path.insert(0, GOLD)
    from make_ref_fixtures import digest, truth_table_inputs
    fx = np.load(os.path.join(GOLD, "ref_bootstrap_p0.npz"))
    x, y, g, c1, c2 = truth_table_inputs(keys0)
    assert digest(c1, c2) == fx["inputs_sha256"].item().decode()
    out, failed = keys0.oracle.eval_bootstrap_batch(c1, c2, g, keys0.btkey, keys0.kskey)
    assert failed == 0
    assert np.array_equal(out, fx["out"].astype(np.uint64))
    truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
    assert np.array_equal(keys0.decrypt(out), truth)


def test_oracle_equals_reference_outputs_wide(F, keys1):
    """The 64-bit set (N = 2048, Q < 2^54, BG 2^9 x 6, Bks 25 x 12): the
    oracle's eval_bootstrap, LWE_keyswitch and LWE_modswitch give exactly the
    reference's words (ref_bootstrap_p1.npz, tests/golden/make_ref_fixtures.py):
    the truth tables at n = 32 and four gates at the full n = 630."""
    import sys
    sys.path.insert(0, GOLD)
    from make_ref_fixtures import digest, full_inputs, keys_digest, truth_table_inputs
    from conftest import KeySet
    fx = np.load(os.path.join(GOLD, "ref_bootstrap_p1.npz"))
    small = KeySet(F, 1, n=int(fx["n_small"]))
    assert keys_digest(small) == fx["keys_sha256"].item().decode()
    x, y, g, c1, c2 = truth_table_inputs(small)
    assert digest(c1, c2) == fx["inputs_sha256"].item().decode()
    out, failed = small.oracle.eval_bootstrap_batch(c1, c2, g, small.btkey, small.kskey)
    assert failed == 0
    assert np.array_equal(out, fx["out"].astype(np.uint64))
    truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
    assert np.array_equal(small.decrypt(out), truth)
    ks_out = np.stack([small.oracle.lwe_keyswitch(r, small.kskey) for r in fx["ks_in"]])
    assert np.array_equal(ks_out, fx["ks_out"])
    ms_out = np.stack([small.oracle.lwe_modswitch(v) for v in fx["ms_in"]])
    assert np.array_equal(ms_out, fx["ms_out"])
    # the full dimension
    assert keys_digest(keys1) == fx["full_keys_sha256"].item().decode()
    fx_, fy, fg, f1, f2 = full_inputs(keys1)
    assert digest(f1, f2) == fx["full_inputs_sha256"].item().decode()
    fout, failed = keys1.oracle.eval_bootstrap_batch(f1, f2, fg, keys1.btkey, keys1.kskey)
    assert failed == 0
    assert np.array_equal(fout, fx["full_out"].astype(np.uint64))


def test_wide_preset_oracle_bootstrap(F, keys1):
    """Preset 1 keys from the host generator bootstrap correctly in the oracle
    (N=2048, Q < 2^54, BG 2^9 x 6)."""
    x = np.array([1, 0], dtype=np.uint8)
    y = np.array([1, 1], dtype=np.uint8)
    c = keys1.encrypt(np.concatenate([x, y]), seed=3)
    out, failed = keys1.oracle.eval_bootstrap_batch(c[:2], c[2:], [F.NAND, F.XOR], keys1.btkey, keys1.kskey)
    assert failed == 0
    assert np.array_equal(keys1.decrypt(out), [0, 1])


def test_container_roundtrip_and_checks(F, keys0, tmp_path):
    """Keys and ciphertexts written to the on-disk container read back word for
    word; another kind, parameter set or a flipped byte is refused."""
    P = keys0.P
    path = str(tmp_path / "kskey.fheacc")
    F.save(path, F.KIND_LWE_KS_KEY, P, keys0.kskey)
    assert np.array_equal(F.load(path, F.KIND_LWE_KS_KEY, P), keys0.kskey)
    ct = keys0.encrypt(np.array([1, 0, 1], dtype=np.uint8))
    cpath = str(tmp_path / "ct.fheacc")
    F.save(cpath, F.KIND_LWE_CT, P, ct)
    back = F.load(cpath, F.KIND_LWE_CT, P).reshape(3, P.n + 1)
    assert np.array_equal(keys0.decrypt(back), [1, 0, 1])
    with pytest.raises(F.FheaccError) as e:
        F.load(cpath, F.KIND_LWE_KS_KEY, P)           # wrong kind
    assert e.value.code == F.EINVAL
    other = F.params_preset(2)
    with pytest.raises(F.FheaccError):
        F.load(cpath, F.KIND_LWE_CT, other)           # other parameter set
    raw = bytearray(open(cpath, "rb").read())
    raw[64 + 17] ^= 0x40
    open(cpath, "wb").write(bytes(raw))
    with pytest.raises(F.FheaccError) as e:
        F.load(cpath, F.KIND_LWE_CT, P)               # corrupted payload
    assert e.value.code == F.EIO


def test_keyswitch_digit_quotients_exact(F):
    """The 64-bit tiled key switch takes each base-Bks digit's quotient as
    floor(a m / 2^64) with m = ceil(2^64 / Bks), which equals floor(a / Bks)
    whenever a (m Bks - 2^64) < 2^64: true for every word below Q of the
    64-bit preset. Checked on the extreme words and random ones, digit by digit
    as the kernel walks them (the quotient becomes the next word)."""
    import random
    P = F.params_preset(1)
    Q, B = int(P.Q), int(P.Bks)
    m = ((1 << 64) - 1) // B + 1
    assert Q * (m * B - (1 << 64)) < (1 << 64)
    rng = random.Random(5)
    words = [0, 1, B - 1, B, Q - 1, Q // 2, Q - B] + [rng.randrange(Q) for _ in range(20000)]
    for a in words:
        for _ in range(int(P.digitKS)):
            q = (a * m) >> 64
            assert q == a // B and a - q * B == a % B
            a = q
