"""Every instantiation of the 32-bit blind-rotation kernel on the GPU, against
the oracle: digitG = 2, 3 and 4 (the last digit taken from the accumulator),
each with 1 (both register budgets), 2 and 3 pipelines per CTA, and a gadget
base above the digit-table limit. Parameter validation rejects gadgets with BG^digitG <= Q, so those need
no kernel. Small n keeps key generation and the oracle quick."""
import numpy as np
import pytest

from conftest import random_gate_batch

pytestmark = pytest.mark.gpu


class SmallSet:
    def __init__(self, F, bg_bits, digit_g, n=24, seed=50):
        P = F.params_preset(0)
        P.n, P.BG_bits, P.digitG = n, bg_bits, digit_g
        F.derive(P)
        self.P, self.F = P, F
        self.lwe_sk = F.LWE_secretkey(P, seed)
        self.rlwe_sk = F.RLWE_secretkey(P, seed + 1)
        self.btkey = F.bootstrap_key(P, seed + 2, self.lwe_sk, self.rlwe_sk)
        self.kskey = F.keyswitch_key(P, seed + 3, self.rlwe_sk, self.lwe_sk)
        from oracle_lib import Oracle
        self.oracle = Oracle.from_params(P)

    def encrypt(self, bits, seed=16):
        return self.F.LWE_encrypt(self.P, seed, self.lwe_sk, bits)

    def decrypt(self, ct):
        return self.F.LWE_decrypt(self.P, self.lwe_sk, ct)


# (BG bits, digits, gates decrypt): a 2^14 base (no digit tables) adds too
# much noise to decrypt at this n
@pytest.mark.parametrize("bg_bits,digit_g,decrypts", [(14, 2, False), (9, 3, True), (7, 4, True)])
def test_kernel_instantiations(F, cuda_ok, bg_bits, digit_g, decrypts):
    ks = SmallSet(F, bg_bits, digit_g)
    assert ks.P.Q >> (bg_bits * digit_g) == 0
    x, y, g, c1, c2 = random_gate_batch(ks, 40, seed=bg_bits)
    ctx = F.Context(ks.P, 0)
    try:
        ctx.upload_bootstrap_key(ks.btkey)
        ctx.upload_keyswitch_key(ks.kskey)
        outs = []
        # every launch shape: 1 pipeline per CTA with the register budget of 2
        # or 3 CTAs per SM, 2 and 3 pipelines per CTA
        for pipes, regs3 in ((1, 0), (1, 1), (2, -1), (3, -1)):
            ctx.set_option(F.OPT_BR_PIPES, pipes)
            ctx.set_option(F.OPT_BR_REGS_FOR_3, regs3)
            outs.append(ctx.eval_bootstrap_batch(c1, c2, g))
    finally:
        ctx.close()
    want, failed = ks.oracle.eval_bootstrap_batch(c1, c2, g, ks.btkey, ks.kskey)
    assert failed == 0
    for out in outs:
        assert np.array_equal(out, want)
    if decrypts:
        truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
        assert np.array_equal(ks.decrypt(outs[0]), truth)
