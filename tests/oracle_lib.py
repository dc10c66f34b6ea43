"""ctypes access to the test libraries: oracle/liboracle.so (the C
restatement of the reference path) and, where it was built, oracle/_ref/libref.so
(the reference's own runtime). Test infrastructure only."""
import ctypes
import importlib
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle.so")
REF_LIB = os.path.join(ORACLE_DIR, "_ref", "libref.so")

_u64p = ctypes.POINTER(ctypes.c_uint64)
_i32p = ctypes.POINTER(ctypes.c_int32)


def pkg():
    import sys
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    return importlib.import_module("3rd_gen_fhe_acc_gb300")


ORACLE_SOURCES = ["fhe_oracle.c", "fhe_keygen.c"]


def build_oracle():
    srcs = [os.path.join(ORACLE_DIR, s) for s in ORACLE_SOURCES]
    deps = srcs + [os.path.join(ORACLE_DIR, "fhe_oracle.h")]
    if not os.path.exists(ORACLE_LIB) or any(os.path.getmtime(ORACLE_LIB) < os.path.getmtime(d) for d in deps):
        subprocess.check_call(["gcc", "-O3", "-fPIC", "-shared", "-pthread"] + srcs + ["-lm", "-o",
                                                                                       ORACLE_LIB + ".tmp"])
        os.replace(ORACLE_LIB + ".tmp", ORACLE_LIB)
    return ORACLE_LIB


class OraParams(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int), ("q", ctypes.c_uint64), ("N", ctypes.c_int), ("Q", ctypes.c_uint64),
        ("BGbits", ctypes.c_uint64), ("digitG", ctypes.c_uint64), ("Br", ctypes.c_uint64),
        ("digitR", ctypes.c_uint64), ("Bks", ctypes.c_uint64), ("digitKS", ctypes.c_uint64),
        ("Bks_R_bits", ctypes.c_uint64), ("digitKS_R", ctypes.c_uint64),
        ("gate_constant", ctypes.c_uint64 * 6),
        ("iN", ctypes.c_uint64), ("ROU", ctypes.c_uint64),
        ("rou", _u64p), ("irou", _u64p), ("digitN", ctypes.c_int), ("rot_bwd", _u64p),
        ("rot_fwd", _u64p),
    ]


def p64(a):
    assert a.dtype == np.uint64 and a.flags.c_contiguous
    return a.ctypes.data_as(_u64p)


class Oracle:
    """The C restatement bound to one parameter set."""

    def __init__(self, n, q, N, Q, BGbits, digitG, Br, digitR, Bks, digitKS, Bks_R_bits, digitKS_R,
                 gate_constant=None):
        L = ctypes.CDLL(build_oracle())
        self.L = L
        for name, res, args in [
            ("ora_params_setup", ctypes.c_int, [ctypes.POINTER(OraParams)]),
            ("ora_params_free", None, [ctypes.POINTER(OraParams)]),
            ("ora_find_Q", ctypes.c_uint64, [ctypes.c_int, ctypes.c_int]),
            ("ora_root_of_unity", ctypes.c_uint64, [ctypes.c_int, ctypes.c_uint64]),
            ("ora_ntt", None, [_u64p, ctypes.c_int, ctypes.c_uint64, _u64p]),
            ("ora_intt", None, [_u64p, ctypes.c_int, ctypes.c_uint64, _u64p, ctypes.c_uint64]),
            ("ora_digit_decompose", None, [ctypes.POINTER(OraParams), _u64p, ctypes.c_uint64, ctypes.c_uint64,
                                           ctypes.c_uint64, _u64p]),
            ("ora_rlwe_mult_rgsw", None, [ctypes.POINTER(OraParams), _u64p, _u64p, _u64p]),
            ("ora_acc_initialization", None, [ctypes.POINTER(OraParams), ctypes.c_uint64, ctypes.c_uint64,
                                              ctypes.c_uint64, ctypes.c_uint64, _u64p]),
            ("ora_blind_rotate", ctypes.c_int, [ctypes.POINTER(OraParams), _u64p, _u64p, ctypes.c_int, _u64p,
                                                ctypes.c_int, _u64p]),
            ("ora_lwe_keyswitch", None, [ctypes.POINTER(OraParams), _u64p, _u64p, _u64p]),
            ("ora_lwe_modswitch", None, [ctypes.POINTER(OraParams), _u64p, _u64p]),
            ("ora_eval_bootstrap", ctypes.c_int, [ctypes.POINTER(OraParams), _u64p, _u64p, ctypes.c_int, _u64p,
                                                  _u64p, ctypes.c_int, _u64p]),
            ("ora_eval_bootstrap_batch", ctypes.c_int, [ctypes.POINTER(OraParams), _u64p, _u64p, _i32p,
                                                        ctypes.c_size_t, _u64p, _u64p, ctypes.c_int, ctypes.c_int,
                                                        _u64p]),
            ("ora_lwe_decrypt", ctypes.c_uint64, [ctypes.POINTER(OraParams), _u64p, _u64p, ctypes.c_uint64]),
            ("ora_poly_substitute", None, [_u64p, ctypes.c_int, ctypes.c_int, ctypes.c_uint64, _u64p]),
            ("ora_rlwe_substitute", None, [ctypes.POINTER(OraParams), _u64p, ctypes.c_int, _u64p]),
            ("ora_rlwe_keyswitch", None, [ctypes.POINTER(OraParams), _u64p, _u64p, _u64p]),
            ("ora_expand_rlwe", None, [ctypes.POINTER(OraParams), _u64p, _u64p, _u64p]),
            ("ora_cmux", None, [ctypes.POINTER(OraParams), _u64p, _u64p, _u64p, _u64p]),
            ("ora_rlwe_blind_rotate", None, [ctypes.POINTER(OraParams), _u64p, ctypes.c_int, _u64p, _u64p]),
            ("ora_homo_expand", None, [ctypes.POINTER(OraParams), _u64p, _u64p, _u64p, _u64p]),
            ("ora_keygen_lwe_sk", ctypes.c_int, [ctypes.POINTER(OraParams), ctypes.c_uint64, _u64p]),
            ("ora_keygen_rlwe_sk", ctypes.c_int, [ctypes.POINTER(OraParams), ctypes.c_uint64, _u64p]),
            ("ora_keygen_bootstrap_key", ctypes.c_int, [ctypes.POINTER(OraParams), ctypes.c_uint64, ctypes.c_uint64,
                                                        _u64p, _u64p, _u64p, ctypes.c_int]),
            ("ora_keygen_lwe_ks_key", ctypes.c_int, [ctypes.POINTER(OraParams), ctypes.c_uint64, ctypes.c_uint64,
                                                     _u64p, _u64p, _u64p, ctypes.c_int]),
            ("ora_lwe_encrypt", ctypes.c_int, [ctypes.POINTER(OraParams), ctypes.c_uint64, ctypes.c_uint64, _u64p,
                                               ctypes.POINTER(ctypes.c_uint8), ctypes.c_size_t, _u64p]),
        ]:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        p = OraParams()
        p.n, p.q, p.N, p.Q = n, q, N, Q
        p.BGbits, p.digitG, p.Br, p.digitR = BGbits, digitG, Br, digitR
        p.Bks, p.digitKS, p.Bks_R_bits, p.digitKS_R = Bks, digitKS, Bks_R_bits, digitKS_R
        gc = gate_constant or [5 * (q >> 3), 7 * (q >> 3), q >> 3, 3 * (q >> 3), 5 * (q >> 3), q >> 3]
        for i in range(6):
            p.gate_constant[i] = gc[i]
        assert L.ora_params_setup(ctypes.byref(p)) == 0
        self.p = p

    # The measured parameter sets, stated without the product (the CPU
    # reference arm of bench.py builds its oracle from these):
    # 0: n=500, N=1024, Q = largest prime < 2^27 with Q = 1 mod 2N, BG=2^7;
    # 1: n=630, N=2048, Q < 2^54, BG=2^9; both q=512, Br=23, Bks=25, Bks_R=2^9.
    PRESETS = {0: dict(n=500, q=512, N=1024, nbit=27, BGbits=7, Br=23, Bks=25, Bks_R_bits=9),
               1: dict(n=630, q=512, N=2048, nbit=54, BGbits=9, Br=23, Bks=25, Bks_R_bits=9)}

    @classmethod
    def preset(cls, k, n=None):
        """A preset with the reference's derivations (digit counts as the
        smallest that cover the modulus, fhe_wo_fpga.cpp:89-161)."""
        d = dict(cls.PRESETS[k])
        if n is not None:
            d["n"] = n
        L = ctypes.CDLL(build_oracle())
        L.ora_find_Q.restype = ctypes.c_uint64
        L.ora_find_Q.argtypes = [ctypes.c_int, ctypes.c_int]
        Q = L.ora_find_Q(d["nbit"], d["N"])

        def digits(base, mod):
            c, v = 0, 1
            while v < mod:
                v *= base
                c += 1
            return c
        return cls(d["n"], d["q"], d["N"], Q, d["BGbits"], digits(1 << d["BGbits"], Q), d["Br"],
                   digits(d["Br"], d["q"]), d["Bks"], digits(d["Bks"], Q), d["Bks_R_bits"],
                   digits(1 << d["Bks_R_bits"], Q))

    @classmethod
    def from_params(cls, P):
        """From a product Params (fheacc_params) of the same set."""
        return cls(P.n, P.q, P.N, P.Q, P.BG_bits, P.digitG, P.Br, P.digitR, P.Bks, P.digitKS, P.Bks_R_bits,
                   P.digitKS_R, list(P.gate_constant))

    def __del__(self):
        try:
            self.L.ora_params_free(ctypes.byref(self.p))
        except Exception:
            pass

    @property
    def N(self):
        return self.p.N

    @property
    def n(self):
        return self.p.n

    def tables(self):
        N = self.p.N
        rou = np.ctypeslib.as_array(self.p.rou, shape=(N,)).copy()
        irou = np.ctypeslib.as_array(self.p.irou, shape=(N,)).copy()
        return rou, irou

    def ntt(self, a):
        a = np.array(a, dtype=np.uint64)
        self.L.ora_ntt(p64(a), self.p.N, self.p.Q, self.p.rou)
        return a

    def intt(self, a):
        a = np.array(a, dtype=np.uint64)
        self.L.ora_intt(p64(a), self.p.N, self.p.Q, self.p.irou, self.p.iN)
        return a

    def digit_decompose(self, rlwe, length, bits):
        out = np.zeros(length * 2 * self.N, dtype=np.uint64)
        rlwe = np.ascontiguousarray(rlwe, dtype=np.uint64)
        self.L.ora_digit_decompose(ctypes.byref(self.p), p64(rlwe), length, (1 << bits) - 1, bits, p64(out))
        return out.reshape(length, 2, self.N)

    def rlwe_mult_rgsw(self, acc, rgsw):
        out = np.zeros(2 * self.N, dtype=np.uint64)
        self.L.ora_rlwe_mult_rgsw(ctypes.byref(self.p), p64(np.ascontiguousarray(acc, dtype=np.uint64)),
                                  p64(np.ascontiguousarray(rgsw, dtype=np.uint64)), p64(out))
        return out

    def acc_initialization(self, embed, b1, b2, value):
        out = np.zeros(2 * self.N, dtype=np.uint64)
        self.L.ora_acc_initialization(ctypes.byref(self.p), embed, b1, b2, value, p64(out))
        return out

    def blind_rotate(self, c1, c2, gate, btkey, fpga_compat=False):
        out = np.zeros(2 * self.N, dtype=np.uint64)
        steps = self.L.ora_blind_rotate(ctypes.byref(self.p), p64(np.ascontiguousarray(c1, dtype=np.uint64)),
                                        p64(np.ascontiguousarray(c2, dtype=np.uint64)), gate, p64(btkey),
                                        int(fpga_compat), p64(out))
        return out, steps

    def lwe_keyswitch(self, rlwe, kskey):
        out = np.zeros(self.n + 1, dtype=np.uint64)
        self.L.ora_lwe_keyswitch(ctypes.byref(self.p), p64(np.ascontiguousarray(rlwe, dtype=np.uint64)),
                                 p64(kskey), p64(out))
        return out

    def lwe_modswitch(self, c):
        out = np.zeros(self.n + 1, dtype=np.uint64)
        self.L.ora_lwe_modswitch(ctypes.byref(self.p), p64(np.ascontiguousarray(c, dtype=np.uint64)), p64(out))
        return out

    def eval_bootstrap(self, c1, c2, gate, btkey, kskey, fpga_compat=False):
        out = np.zeros(self.n + 1, dtype=np.uint64)
        rc = self.L.ora_eval_bootstrap(ctypes.byref(self.p), p64(np.ascontiguousarray(c1, dtype=np.uint64)),
                                       p64(np.ascontiguousarray(c2, dtype=np.uint64)), gate, p64(btkey),
                                       p64(kskey), int(fpga_compat), p64(out))
        return out, rc

    def eval_bootstrap_batch(self, c1, c2, gates, btkey, kskey, fpga_compat=False, threads=0):
        c1 = np.ascontiguousarray(c1, dtype=np.uint64).reshape(-1, self.n + 1)
        c2 = np.ascontiguousarray(c2, dtype=np.uint64).reshape(-1, self.n + 1)
        g = np.ascontiguousarray(np.asarray(gates, dtype=np.int32).reshape(-1))
        if g.size == 1 and c1.shape[0] > 1:
            g = np.full(c1.shape[0], g[0], dtype=np.int32)
        out = np.zeros_like(c1)
        failed = self.L.ora_eval_bootstrap_batch(ctypes.byref(self.p), p64(c1), p64(c2), g.ctypes.data_as(_i32p),
                                                 c1.shape[0], p64(btkey), p64(kskey), int(fpga_compat), threads,
                                                 p64(out))
        return out, failed

    def keygen(self, seed, threads=0, E_rlwe=18):
        """(lwe_sk, rlwe_sk_ntt, btkey, kskey) from the oracle's own seeded
        generator (fhe_keygen.c), in the reference's layouts."""
        p = self.p
        threads = threads or os.cpu_count() or 1
        lsk = np.zeros(p.n, dtype=np.uint64)
        rsk = np.zeros(p.N, dtype=np.uint64)
        assert self.L.ora_keygen_lwe_sk(ctypes.byref(p), seed, p64(lsk)) == 0
        assert self.L.ora_keygen_rlwe_sk(ctypes.byref(p), seed + 1, p64(rsk)) == 0
        bt = np.zeros(p.Br * p.digitR * p.n * p.digitG * 4 * p.N, dtype=np.uint64)
        ks = np.zeros(p.Bks * p.digitKS * p.N * (p.n + 1), dtype=np.uint64)
        self.L.ora_keygen_bootstrap_key(ctypes.byref(p), seed + 2, E_rlwe, p64(lsk), p64(rsk), p64(bt), threads)
        self.L.ora_keygen_lwe_ks_key(ctypes.byref(p), seed + 3, E_rlwe, p64(rsk), p64(lsk), p64(ks), threads)
        return lsk, rsk, bt, ks

    def lwe_encrypt(self, seed, sk, bits):
        """LWE_encrypt (t = 4, E = q/16) of each bit: [count][n+1]."""
        bits = np.ascontiguousarray(bits, dtype=np.uint8)
        out = np.zeros((bits.size, self.p.n + 1), dtype=np.uint64)
        self.L.ora_lwe_encrypt(ctypes.byref(self.p), seed, self.p.q // 16, p64(np.ascontiguousarray(sk)),
                               bits.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), bits.size, p64(out))
        return out

    def lwe_decrypt(self, sk, c, t=4):
        return self.L.ora_lwe_decrypt(ctypes.byref(self.p), p64(np.ascontiguousarray(sk, dtype=np.uint64)),
                                      p64(np.ascontiguousarray(c, dtype=np.uint64)), t)

    def rlwe_substitute(self, c, f):
        out = np.zeros(2 * self.N, dtype=np.uint64)
        self.L.ora_rlwe_substitute(ctypes.byref(self.p), p64(np.ascontiguousarray(c, dtype=np.uint64)), f, p64(out))
        return out

    def rlwe_keyswitch(self, c, ksk):
        out = np.zeros(2 * self.N, dtype=np.uint64)
        self.L.ora_rlwe_keyswitch(ctypes.byref(self.p), p64(np.ascontiguousarray(c, dtype=np.uint64)),
                                  p64(np.ascontiguousarray(ksk, dtype=np.uint64)), p64(out))
        return out

    def expand_rlwe(self, c, subs_key):
        out = np.zeros(self.N * 2 * self.N, dtype=np.uint64)
        self.L.ora_expand_rlwe(ctypes.byref(self.p), p64(np.ascontiguousarray(c, dtype=np.uint64)),
                               p64(np.ascontiguousarray(subs_key, dtype=np.uint64)), p64(out))
        return out.reshape(self.N, 2 * self.N)

    def cmux(self, c0, c1, sel):
        out = np.zeros(2 * self.N, dtype=np.uint64)
        self.L.ora_cmux(ctypes.byref(self.p), *(p64(np.ascontiguousarray(x, dtype=np.uint64)) for x in (c0, c1, sel)),
                        p64(out))
        return out

    def rlwe_blind_rotate(self, c, forward, rgsws):
        out = np.zeros(2 * self.N, dtype=np.uint64)
        self.L.ora_rlwe_blind_rotate(ctypes.byref(self.p), p64(np.ascontiguousarray(c, dtype=np.uint64)),
                                     1 if forward else 0, p64(np.ascontiguousarray(rgsws, dtype=np.uint64)),
                                     p64(out))
        return out

    def homo_expand(self, packed, enc_sec, subs_key):
        dG = int(self.p.digitG)
        out = np.zeros(self.N * dG * 4 * self.N, dtype=np.uint64)
        self.L.ora_homo_expand(ctypes.byref(self.p), p64(np.ascontiguousarray(packed, dtype=np.uint64)),
                               p64(np.ascontiguousarray(enc_sec, dtype=np.uint64)),
                               p64(np.ascontiguousarray(subs_key, dtype=np.uint64)), p64(out))
        return out.reshape(self.N, dG * 4 * self.N)


class RefParams(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int), ("q", ctypes.c_uint64), ("N", ctypes.c_int), ("Q", ctypes.c_uint64),
        ("BGbits", ctypes.c_uint64), ("digitG", ctypes.c_uint64), ("Br", ctypes.c_uint64),
        ("digitR", ctypes.c_uint64), ("Bks", ctypes.c_uint64), ("digitKS", ctypes.c_uint64),
        ("Bks_R_bits", ctypes.c_uint64), ("digitKS_R", ctypes.c_uint64),
        ("gate_constant", ctypes.c_uint64 * 6), ("iN", ctypes.c_uint64), ("ROU", ctypes.c_uint64),
    ]


def ref_available():
    return os.path.exists(REF_LIB)


class Ref:
    """The reference's own runtime (oracle/_ref/libref.so), one process-wide
    parameter set (the reference keeps its parameters in globals)."""

    def __init__(self, ora):
        L = ctypes.CDLL(REF_LIB)
        self.L = L
        vp = None
        for name, res, args in [
            ("ref_setup", ctypes.c_int, [ctypes.POINTER(RefParams)]),
            ("ref_find_Q", ctypes.c_uint64, [ctypes.c_int, ctypes.c_int]),
            ("ref_ntt", vp, [_u64p]), ("ref_intt", vp, [_u64p]), ("ref_tables", vp, [_u64p, _u64p]),
            ("ref_rlwe_mult_rgsw", vp, [_u64p, _u64p, _u64p]),
            ("ref_acc_initialization", vp, [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                            _u64p]),
            ("ref_load_keys", vp, [_u64p, _u64p]), ("ref_free_keys", vp, []),
            ("ref_eval_bootstrap", ctypes.c_int, [_u64p, _u64p, ctypes.c_int, _u64p]),
            ("ref_lwe_keyswitch", vp, [_u64p, _u64p]), ("ref_lwe_modswitch", vp, [_u64p, _u64p]),
            ("ref_rlwe_substitute", vp, [_u64p, ctypes.c_int, _u64p]),
            ("ref_rlwe_keyswitch", vp, [_u64p, _u64p, _u64p]),
            ("ref_expand_rlwe", vp, [_u64p, _u64p, _u64p]),
            ("ref_cmux", vp, [_u64p, _u64p, _u64p, _u64p]),
            ("ref_blind_rotate", ctypes.c_int, [_u64p, ctypes.c_int, _u64p, ctypes.c_int, _u64p]),
            ("ref_homo_expand", vp, [_u64p, _u64p, _u64p, _u64p]),
        ]:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        o = ora.p
        p = RefParams()
        p.n, p.q, p.N, p.Q = o.n, o.q, o.N, o.Q
        p.BGbits, p.digitG, p.Br, p.digitR = o.BGbits, o.digitG, o.Br, o.digitR
        p.Bks, p.digitKS, p.Bks_R_bits, p.digitKS_R = o.Bks, o.digitKS, o.Bks_R_bits, o.digitKS_R
        for i in range(6):
            p.gate_constant[i] = o.gate_constant[i]
        assert L.ref_setup(ctypes.byref(p)) == 0
        self.p = p
        self.N, self.n = o.N, o.n

    def tables(self):
        rou = np.zeros(self.N, dtype=np.uint64)
        irou = np.zeros(self.N, dtype=np.uint64)
        self.L.ref_tables(p64(rou), p64(irou))
        return rou, irou

    def ntt(self, a):
        a = np.array(a, dtype=np.uint64)
        self.L.ref_ntt(p64(a))
        return a

    def intt(self, a):
        a = np.array(a, dtype=np.uint64)
        self.L.ref_intt(p64(a))
        return a

    def rlwe_mult_rgsw(self, acc, rgsw):
        out = np.zeros(2 * self.N, dtype=np.uint64)
        self.L.ref_rlwe_mult_rgsw(p64(np.ascontiguousarray(acc, dtype=np.uint64)),
                                  p64(np.ascontiguousarray(rgsw, dtype=np.uint64)), p64(out))
        return out

    def acc_initialization(self, embed, b1, b2, value):
        out = np.zeros(2 * self.N, dtype=np.uint64)
        self.L.ref_acc_initialization(embed, b1, b2, value, p64(out))
        return out

    def load_keys(self, btkey, kskey):
        self.L.ref_load_keys(p64(btkey), p64(kskey))

    def free_keys(self):
        self.L.ref_free_keys()

    def eval_bootstrap(self, c1, c2, gate):
        out = np.zeros(self.n + 1, dtype=np.uint64)
        rc = self.L.ref_eval_bootstrap(p64(np.ascontiguousarray(c1, dtype=np.uint64)),
                                       p64(np.ascontiguousarray(c2, dtype=np.uint64)), gate, p64(out))
        return out, rc

    def lwe_keyswitch(self, rlwe):
        out = np.zeros(self.n + 1, dtype=np.uint64)
        self.L.ref_lwe_keyswitch(p64(np.ascontiguousarray(rlwe, dtype=np.uint64)), p64(out))
        return out

    def lwe_modswitch(self, c):
        out = np.zeros(self.n + 1, dtype=np.uint64)
        self.L.ref_lwe_modswitch(p64(np.ascontiguousarray(c, dtype=np.uint64)), p64(out))
        return out

    def rlwe_substitute(self, c, f):
        out = np.zeros(2 * self.N, dtype=np.uint64)
        self.L.ref_rlwe_substitute(p64(np.ascontiguousarray(c, dtype=np.uint64)), f, p64(out))
        return out

    def rlwe_keyswitch(self, c, ksk):
        out = np.zeros(2 * self.N, dtype=np.uint64)
        self.L.ref_rlwe_keyswitch(p64(np.ascontiguousarray(c, dtype=np.uint64)),
                                  p64(np.ascontiguousarray(ksk, dtype=np.uint64)), p64(out))
        return out

    def expand_rlwe(self, c, subs):
        out = np.zeros(self.N * 2 * self.N, dtype=np.uint64)
        self.L.ref_expand_rlwe(p64(np.ascontiguousarray(c, dtype=np.uint64)),
                               p64(np.ascontiguousarray(subs, dtype=np.uint64)), p64(out))
        return out.reshape(self.N, 2 * self.N)

    def cmux(self, c0, c1, sel):
        out = np.zeros(2 * self.N, dtype=np.uint64)
        self.L.ref_cmux(*(p64(np.ascontiguousarray(x, dtype=np.uint64)) for x in (c0, c1, sel)), p64(out))
        return out

    def blind_rotate(self, c, forward, rgsws, count):
        out = np.zeros(2 * self.N, dtype=np.uint64)
        rc = self.L.ref_blind_rotate(p64(np.ascontiguousarray(c, dtype=np.uint64)), 1 if forward else 0,
                                     p64(np.ascontiguousarray(rgsws, dtype=np.uint64)), count, p64(out))
        return out, rc

    def homo_expand(self, packed, enc_sec, subs):
        dG = int(self.p.digitG)
        out = np.zeros(self.N * dG * 4 * self.N, dtype=np.uint64)
        self.L.ref_homo_expand(*(p64(np.ascontiguousarray(x, dtype=np.uint64)) for x in (packed, enc_sec, subs)),
                               p64(out))
        return out.reshape(self.N, dG * 4 * self.N)
