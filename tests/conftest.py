import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

from oracle_lib import Oracle, pkg  # noqa: E402

# seeds of the shared key set (deterministic on every machine)
SEEDS = dict(lwe_sk=11, rlwe_sk=12, btkey=13, kskey=14, subs=15, enc=16)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")
    config.addinivalue_line("markers", "slow: takes more than ~30 s on the CPU")


@pytest.fixture(scope="session")
def F():
    """The product package (libfheacc.so must be built)."""
    import __graft_entry__
    __graft_entry__.build_product()
    return pkg()


class KeySet:
    def __init__(self, F, preset, n=None):
        """The shared key set of a preset; n: a reduced LWE dimension (the
        per-step work is unchanged, key generation and the oracle are quick)."""
        self.P = F.params_preset(preset)
        P = self.P
        if n is not None:
            P.n = n
            F.derive(P)
        self.lwe_sk = F.LWE_secretkey(P, SEEDS["lwe_sk"])
        self.rlwe_sk = F.RLWE_secretkey(P, SEEDS["rlwe_sk"])
        self.btkey = F.bootstrap_key(P, SEEDS["btkey"], self.lwe_sk, self.rlwe_sk)
        self.kskey = F.keyswitch_key(P, SEEDS["kskey"], self.rlwe_sk, self.lwe_sk)
        self._subs = None
        self.F = F
        self.oracle = Oracle.from_params(P)

    @property
    def subs(self):
        if self._subs is None:
            self._subs = self.F.substitute_key(self.P, SEEDS["subs"], self.rlwe_sk)
        return self._subs

    def encrypt(self, bits, seed=SEEDS["enc"]):
        return self.F.LWE_encrypt(self.P, seed, self.lwe_sk, bits)

    def decrypt(self, ct):
        return self.F.LWE_decrypt(self.P, self.lwe_sk, ct)


@pytest.fixture(scope="session")
def keys0(F):
    """Preset 0 (N=1024, Q < 2^27, BG 2^7 x 4, n=500) key set."""
    return KeySet(F, 0)


@pytest.fixture(scope="session")
def keys1(F):
    """Preset 1 (N=2048, Q < 2^54, BG 2^9 x 6, n=630) key set; the bootstrap
    key is 11.4 GB of host memory."""
    return KeySet(F, 1)


@pytest.fixture(scope="session")
def cuda_ok():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="session")
def ctx0(F, keys0, cuda_ok):
    ctx = F.Context(keys0.P, 0)
    ctx.upload_bootstrap_key(keys0.btkey)
    ctx.upload_keyswitch_key(keys0.kskey)
    yield ctx
    ctx.close()


@pytest.fixture(scope="session")
def ctx1(F, keys1, cuda_ok):
    ctx = F.Context(keys1.P, 0)
    ctx.upload_bootstrap_key(keys1.btkey)
    ctx.upload_keyswitch_key(keys1.kskey)
    yield ctx
    ctx.close()


def random_gate_batch(ks, count, seed, gates=None):
    """count independent gate inputs: bits x, y, their encryptions, gate codes."""
    rng = np.random.default_rng(seed)
    x = rng.integers(0, 2, count).astype(np.uint8)
    y = rng.integers(0, 2, count).astype(np.uint8)
    g = rng.integers(0, 6, count).astype(np.int32) if gates is None else np.asarray(gates, dtype=np.int32)
    c = ks.encrypt(np.concatenate([x, y]), seed=1000 + seed)
    return x, y, g, c[:count].copy(), c[count:].copy()


def first_residue(P, c1, c2, gates):
    """Residue of the first blind-rotation step (i = 0, j = 0) of each gate:
    (q - a_0) mod q mod Br, a = LWE_evaluate(c1, c2) (LWE.cpp:203-222)."""
    q = int(P.q)
    a1 = c1[:, 0].astype(np.int64)
    a2 = c2[:, 0].astype(np.int64)
    x2 = (gates == 4) | (gates == 5)
    a = np.where(x2, 2 * (a1 - a2), a1 + a2) % q
    return ((q - a) % q) % int(P.Br)


def x1_gate_batch(ks, count, seed):
    """count gates of which about half have residue 0 at the first step, the
    case where the issue order of fpga_eval_bootstrap_x1 differs from the
    CPU path's (it applies that step's key anyway); drawn from a larger pool
    of random encryptions."""
    x, y, g, c1, c2 = random_gate_batch(ks, 48 * count, seed)
    r0 = first_residue(ks.P, c1, c2, g)
    zero = np.flatnonzero(r0 == 0)[:(count + 1) // 2]
    other = np.flatnonzero(r0 != 0)[:count - len(zero)]
    idx = np.sort(np.concatenate([zero, other]))
    assert len(zero) >= 1 and len(idx) == count
    return x[idx], y[idx], g[idx], c1[idx].copy(), c2[idx].copy(), r0[idx] == 0
