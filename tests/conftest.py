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
    def __init__(self, F, preset):
        self.P = F.params_preset(preset)
        P = self.P
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
