"""GB300 (sm_103a) backend for the FHEW/AP gate-bootstrapping path of
zhehongw/3rd_Gen_FHE_ACC.

Python host side over the C ABI of libfheacc.so (include/fheacc.h). It keeps
the names and the argument meaning of the reference runtime's host API:
key generation (LWE::LWE_secretkey, RLWE::RLWE_secretkey, RLWE::bootstrap_key,
LWE::keyswitch_key, application::substitute_key), LWE_encrypt / LWE_decrypt,
RLWE::eval_bootstrap, and the FPGA backend's fixed-width gate calls
fpga_eval_bootstrap_x1/x4/x8/x12/x16 (FHE_ACC_runtime/include/myfpga.h:287-331),
here served by the GPU. Ciphertexts and keys are numpy uint64 arrays in the
reference's layouts (see include/fheacc.h).

The package imports as importlib.import_module("3rd_gen_fhe_acc_gb300").
The shared library must be built first (build.py, or __graft_entry__.build());
nothing here falls back to a CPU implementation.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfheacc.so")

OR, AND, NOR, NAND, XOR, XNOR = range(6)
GATES = {"OR": OR, "AND": AND, "NOR": NOR, "NAND": NAND, "XOR": XOR, "XNOR": XNOR}
FLAG_FPGA_COMPAT = 1
FLAG_PROFILE = 2
FLAG_FPGA_X1 = 4
NOALLOC_MAX_GATES = 64
OPT_BR_REGS_FOR_3 = 1
OPT_BR_CTAS_PER_SM = 2
OPT_BR_GROUP = 3
OPT_BR_WINDOW = 4
OPT_BR_PIPES = 5
OPT_BR_POOL = 6
OPT_DEBUG_WAIT_LIMIT = 7
OPT_KS_TILED = 8
OPT_BR_SOLO = 9
GRAPH_CONCURRENT = 1
STATUS_WAIT_LIMIT = 1
KIND_LWE_SK, KIND_RLWE_SK, KIND_BOOTSTRAP_KEY, KIND_LWE_KS_KEY, KIND_SUBS_KEY, KIND_LWE_CT, KIND_RLWE_CT, \
    KIND_RGSW_CT = range(1, 9)

OK = 0
EINVAL, ENOMEM, ENODEV, EIO, ETIMEDOUT, ENOKEY, EBUSY, EMISMATCH = -22, -12, -19, -5, -110, -126, -16, -74

_u64p = ctypes.POINTER(ctypes.c_uint64)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u32p = ctypes.POINTER(ctypes.c_uint32)


class Params(ctypes.Structure):
    """fheacc_params (include/fheacc.h); the reference's globals, params.h:11-134."""
    _fields_ = [
        ("n", ctypes.c_int32), ("q", ctypes.c_uint32), ("N", ctypes.c_int32), ("nbit", ctypes.c_uint32),
        ("Q", ctypes.c_uint64),
        ("BG_bits", ctypes.c_uint32), ("digitG", ctypes.c_uint32), ("Br", ctypes.c_uint32),
        ("digitR", ctypes.c_uint32), ("Bks", ctypes.c_uint32), ("digitKS", ctypes.c_uint32),
        ("Bks_R_bits", ctypes.c_uint32), ("digitKS_R", ctypes.c_uint32),
        ("gate_constant", ctypes.c_uint64 * 6),
        ("iN", ctypes.c_uint64), ("ROU", ctypes.c_uint64), ("E", ctypes.c_uint32), ("E_rlwe", ctypes.c_uint32),
    ]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["gate_constant"] = list(self.gate_constant)
        return d


class RequestDone(ctypes.Structure):
    _fields_ = [("request_id", ctypes.c_uint64), ("status", ctypes.c_int32), ("queue_ms", ctypes.c_double),
                ("latency_ms", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("rounds", ctypes.c_uint64), ("gates", ctypes.c_uint64), ("busy_s", ctypes.c_double),
                ("waiting", ctypes.c_uint64), ("active", ctypes.c_uint64), ("free_slots", ctypes.c_uint64),
                ("pool_slots", ctypes.c_uint64), ("lanes", ctypes.c_uint64)]


class TuneTrial(ctypes.Structure):
    _fields_ = [("regs_for_3", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32), ("group", ctypes.c_int32),
                ("window", ctypes.c_int32), ("pipes", ctypes.c_int32), ("ms", ctypes.c_float)]


class FheaccError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("fheacc error %d: %s" % (code, msg))
        self.code = code


_lib = None


def lib():
    """The loaded libfheacc.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FheaccError(ENODEV, "libfheacc.so is not built (run __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER(Params)
        vp = ctypes.c_void_p
        sz = ctypes.c_size_t
        sig = {
            "fheacc_params_preset": (ctypes.c_int, [ctypes.c_int, P]),
            "fheacc_params_derive": (ctypes.c_int, [P]),
            "fheacc_bootstrap_key_words": (sz, [P]),
            "fheacc_lwe_ks_key_words": (sz, [P]),
            "fheacc_subs_key_words": (sz, [P]),
            "fheacc_twiddle_tables": (ctypes.c_int, [P, _u64p, _u64p]),
            "fheacc_keygen_lwe_sk": (ctypes.c_int, [P, ctypes.c_uint64, _u64p]),
            "fheacc_keygen_rlwe_sk": (ctypes.c_int, [P, ctypes.c_uint64, _u64p]),
            "fheacc_keygen_bootstrap_key": (ctypes.c_int, [P, ctypes.c_uint64, _u64p, _u64p, _u64p, ctypes.c_int]),
            "fheacc_keygen_lwe_ks_key": (ctypes.c_int, [P, ctypes.c_uint64, _u64p, _u64p, _u64p, ctypes.c_int]),
            "fheacc_keygen_subs_key": (ctypes.c_int, [P, ctypes.c_uint64, _u64p, _u64p, ctypes.c_int]),
            "fheacc_lwe_encrypt": (ctypes.c_int, [P, ctypes.c_uint64, _u64p, _u8p, sz, _u64p]),
            "fheacc_lwe_decrypt": (ctypes.c_int, [P, _u64p, _u64p, sz, _u8p]),
            "fheacc_rlwe_encrypt": (ctypes.c_int, [P, ctypes.c_uint64, _u64p, _u64p, _u64p]),
            "fheacc_rgsw_encrypt": (ctypes.c_int, [P, ctypes.c_uint64, _u64p, _u64p, _u64p]),
            "fheacc_container_save": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_uint32, P, _u64p, sz]),
            "fheacc_container_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_uint32, P, _u64p, sz]),
            "fheacc_container_info": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint32),
                                                     ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(sz)]),
            "fheacc_cmux_async": (ctypes.c_int, [vp, vp, vp, sz, vp, ctypes.c_int, vp, sz, vp]),
            "fheacc_rlwe_blind_rotate_async": (ctypes.c_int, [vp, vp, vp, ctypes.c_int, vp, sz, vp]),
            "fheacc_homo_expand": (ctypes.c_int, [vp, vp, vp, vp, vp]),
            "fheacc_rlwe_phase": (ctypes.c_int, [P, _u64p, _u64p, _u64p]),
            "fheacc_create": (ctypes.c_int, [P, ctypes.c_int, ctypes.POINTER(vp)]),
            "fheacc_destroy": (ctypes.c_int, [vp]),
            "fheacc_last_error": (ctypes.c_char_p, [vp]),
            "fheacc_get_params": (ctypes.c_int, [vp, P]),
            "fheacc_device_bytes": (sz, [vp]),
            "fheacc_upload_bootstrap_key": (ctypes.c_int, [vp, _u64p, sz]),
            "fheacc_upload_lwe_ks_key": (ctypes.c_int, [vp, _u64p, sz]),
            "fheacc_upload_subs_key": (ctypes.c_int, [vp, _u64p, sz]),
            "fheacc_verify_bootstrap_key": (ctypes.c_int, [vp, _u64p, sz]),
            "fheacc_verify_subs_key": (ctypes.c_int, [vp, _u64p, sz]),
            "fheacc_bootstrap": (ctypes.c_int, [vp, _u64p, _u64p, _i32p, sz, _u64p, ctypes.c_uint32]),
            "fheacc_bootstrap_async": (ctypes.c_int, [vp, vp, vp, vp, sz, vp, ctypes.c_uint32, vp]),
            "fheacc_bootstrap_plain_async": (ctypes.c_int, [vp, vp, vp, vp, sz, vp, ctypes.c_uint32, vp]),
            "fheacc_bootstrap_noalloc": (ctypes.c_int, [vp, vp, vp, vp, sz, vp, ctypes.c_uint32, vp]),
            "fheacc_rlwe_substitute_async": (ctypes.c_int, [vp, vp, sz, ctypes.c_int, vp, vp]),
            "fheacc_rlwe_keyswitch_async": (ctypes.c_int, [vp, vp, sz, vp, vp, vp]),
            "fheacc_subs_keyswitch_async": (ctypes.c_int, [vp, vp, sz, ctypes.c_int, vp, vp]),
            "fheacc_expand_rlwe": (ctypes.c_int, [vp, vp, vp, vp]),
            "fheacc_server_create": (ctypes.c_int, [vp, sz, sz, ctypes.POINTER(vp)]),
            "fheacc_server_submit": (ctypes.c_int, [vp, _u64p, ctypes.c_uint32, _i32p, _u32p, _u32p, ctypes.c_uint32,
                                                    ctypes.c_uint32, _u64p, ctypes.POINTER(ctypes.c_uint64)]),
            "fheacc_server_poll": (ctypes.c_int, [vp, ctypes.POINTER(RequestDone), sz, ctypes.POINTER(sz),
                                                  ctypes.c_uint32]),
            "fheacc_server_stats": (ctypes.c_int, [vp, ctypes.POINTER(ServerStats)]),
            "fheacc_server_destroy": (ctypes.c_int, [vp]),
            "fheacc_ntt_forward": (ctypes.c_int, [vp, vp, sz, vp]),
            "fheacc_ntt_inverse": (ctypes.c_int, [vp, vp, sz, vp]),
            "fheacc_rlwe_mult_rgsw": (ctypes.c_int, [vp, vp, vp, vp, sz, vp]),
            "fheacc_blind_rotate_async": (ctypes.c_int, [vp, vp, vp, vp, sz, vp, ctypes.c_uint32, vp]),
            "fheacc_lwe_keyswitch_async": (ctypes.c_int, [vp, vp, sz, vp, vp]),
            "fheacc_lwe_modswitch_async": (ctypes.c_int, [vp, vp, sz, vp, vp]),
            "fheacc_sync": (ctypes.c_int, [vp, ctypes.c_uint32]),
            "fheacc_device_status": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_uint32)]),
            "fheacc_kernel_launches": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_uint64)]),
            "fheacc_kernel_times": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_float)]),
            "fheacc_set_option": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int]),
            "fheacc_measure_imad_rate": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_double)]),
            "fheacc_measure_components": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_double)]),
            "fheacc_measure_l2_read_rate": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_double)]),
            "fheacc_autotune": (ctypes.c_int, [vp, sz, ctypes.POINTER(TuneTrial), ctypes.c_int,
                                               ctypes.POINTER(ctypes.c_int)]),
            "fheacc_graph_create": (ctypes.c_int, [ctypes.POINTER(vp), ctypes.c_uint32]),
            "fheacc_graph_add_bootstrap": (ctypes.c_int, [vp, vp, vp, vp, vp, sz, vp]),
            "fheacc_graph_launch": (ctypes.c_int, [vp, vp]),
            "fheacc_graph_batches": (sz, [vp]),
            "fheacc_graph_last_error": (ctypes.c_char_p, [vp]),
            "fheacc_graph_destroy": (ctypes.c_int, [vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p64(a):
    assert a.dtype == np.uint64 and a.flags.c_contiguous
    return a.ctypes.data_as(_u64p)


def _check(rc, ctx=None):
    if rc != OK:
        msg = lib().fheacc_last_error(ctx)
        raise FheaccError(rc, msg.decode() if msg else "")


def params_preset(preset=0):
    """Parameter preset 0 (N=1024, Q<2^27, n=500), 1 (N=2048, Q<2^54, n=630) or
    2 (the reference CPU app's set, fhe_wo_fpga.cpp:35-146)."""
    p = Params()
    _check(lib().fheacc_params_preset(preset, ctypes.byref(p)))
    return p


def derive(p):
    _check(lib().fheacc_params_derive(ctypes.byref(p)))
    return p


def bootstrap_key_words(p):
    return lib().fheacc_bootstrap_key_words(ctypes.byref(p))


def lwe_ks_key_words(p):
    return lib().fheacc_lwe_ks_key_words(ctypes.byref(p))


def subs_key_words(p):
    return lib().fheacc_subs_key_words(ctypes.byref(p))


def twiddle_tables(p):
    rou = np.zeros(p.N, dtype=np.uint64)
    irou = np.zeros(p.N, dtype=np.uint64)
    _check(lib().fheacc_twiddle_tables(ctypes.byref(p), _p64(rou), _p64(irou)))
    return rou, irou


# ------------------------------------------------------------ key generation
def LWE_secretkey(p, seed):
    """LWE::LWE_secretkey (LWE.cpp:22-53): n ternary words mod q."""
    sk = np.zeros(p.n, dtype=np.uint64)
    _check(lib().fheacc_keygen_lwe_sk(ctypes.byref(p), seed, _p64(sk)))
    return sk


def RLWE_secretkey(p, seed):
    """RLWE::RLWE_secretkey (RLWE.cpp:243-279): the NTT-domain poly a."""
    sk = np.zeros(p.N, dtype=np.uint64)
    _check(lib().fheacc_keygen_rlwe_sk(ctypes.byref(p), seed, _p64(sk)))
    return sk


def bootstrap_key(p, seed, lwe_sk, rlwe_sk, threads=0):
    """RLWE::bootstrap_key (RLWE.cpp:579-606), layout [Br][digitR][n][digitG][2][2][N]."""
    bt = np.zeros(bootstrap_key_words(p), dtype=np.uint64)
    _check(lib().fheacc_keygen_bootstrap_key(ctypes.byref(p), seed, _p64(lwe_sk), _p64(rlwe_sk), _p64(bt), threads))
    return bt


def keyswitch_key(p, seed, rlwe_sk, lwe_sk, threads=0):
    """LWE::keyswitch_key (LWE.cpp:55-106), layout [Bks][digitKS][N][n+1]."""
    ks = np.zeros(lwe_ks_key_words(p), dtype=np.uint64)
    _check(lib().fheacc_keygen_lwe_ks_key(ctypes.byref(p), seed, _p64(rlwe_sk), _p64(lwe_sk), _p64(ks), threads))
    return ks


def substitute_key(p, seed, rlwe_sk, threads=0):
    """application::substitute_key (app.cpp:4-24), layout [log2 N][digitKS_R][2][N]."""
    sk = np.zeros(subs_key_words(p), dtype=np.uint64)
    _check(lib().fheacc_keygen_subs_key(ctypes.byref(p), seed, _p64(rlwe_sk), _p64(sk), threads))
    return sk


def LWE_encrypt(p, seed, lwe_sk, bits):
    """LWE::LWE_encrypt (LWE.cpp:108-146) of bits with t = 4; [count][n+1]."""
    bits = np.ascontiguousarray(np.asarray(bits, dtype=np.uint8).reshape(-1))
    out = np.zeros((bits.size, p.n + 1), dtype=np.uint64)
    _check(lib().fheacc_lwe_encrypt(ctypes.byref(p), seed, _p64(lwe_sk), bits.ctypes.data_as(_u8p), bits.size,
                                    _p64(out)))
    return out


def LWE_decrypt(p, lwe_sk, ct):
    """LWE::LWE_decrypt (LWE.cpp:148-190), t = 4: values in [0, 4)."""
    ct = np.ascontiguousarray(ct, dtype=np.uint64).reshape(-1, p.n + 1)
    out = np.zeros(ct.shape[0], dtype=np.uint8)
    _check(lib().fheacc_lwe_decrypt(ctypes.byref(p), _p64(lwe_sk), _p64(ct), ct.shape[0], out.ctypes.data_as(_u8p)))
    return out


def RLWE_encrypt(p, seed, rlwe_sk, msg_ntt):
    out = np.zeros(2 * p.N, dtype=np.uint64)
    msg_ntt = np.ascontiguousarray(msg_ntt, dtype=np.uint64)
    _check(lib().fheacc_rlwe_encrypt(ctypes.byref(p), seed, _p64(rlwe_sk), _p64(msg_ntt), _p64(out)))
    return out


def RGSW_encrypt(p, seed, rlwe_sk, msg_ntt):
    """RGSW_ciphertext(m, z) (RLWE.cpp:561-577): [digitG][2][2][N] words."""
    out = np.zeros(p.digitG * 4 * p.N, dtype=np.uint64)
    msg_ntt = np.ascontiguousarray(msg_ntt, dtype=np.uint64)
    _check(lib().fheacc_rgsw_encrypt(ctypes.byref(p), seed, _p64(rlwe_sk), _p64(msg_ntt), _p64(out)))
    return out


def save(path, kind, p, words):
    """Writes words (uint64, any shape) to the on-disk container (fheacc_container_save)."""
    w = np.ascontiguousarray(words, dtype=np.uint64).reshape(-1)
    _check(lib().fheacc_container_save(os.fsencode(path), kind, ctypes.byref(p), _p64(w), w.size))


def load(path, kind, p):
    """Reads a container written by save() for the same kind and parameter set."""
    k, fp, n = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_size_t()
    _check(lib().fheacc_container_info(os.fsencode(path), ctypes.byref(k), ctypes.byref(fp), ctypes.byref(n)))
    out = np.zeros(n.value, dtype=np.uint64)
    _check(lib().fheacc_container_load(os.fsencode(path), kind, ctypes.byref(p), _p64(out), out.size))
    return out


def RLWE_phase(p, rlwe_sk, ct):
    out = np.zeros(p.N, dtype=np.uint64)
    ct = np.ascontiguousarray(ct, dtype=np.uint64)
    _check(lib().fheacc_rlwe_phase(ctypes.byref(p), _p64(rlwe_sk), _p64(ct), _p64(out)))
    return out


def gate_truth(gate, x, y):
    """Plaintext truth table of the reference's gates (test.cpp:496-625)."""
    x = np.asarray(x, dtype=np.uint8)
    y = np.asarray(y, dtype=np.uint8)
    return {OR: x | y, AND: x & y, NOR: (x | y) ^ 1, NAND: (x & y) ^ 1, XOR: x ^ y, XNOR: (x ^ y) ^ 1}[gate]


# ------------------------------------------------------------------ device
class Context:
    """A device context (fheacc_ctx): parameters, twiddles and resident keys.

    Replaces the FPGA slot set-up (OCL_config_wr_rd, BAR1_ROU_table_*_wr,
    dma_write_*; myfpga.cpp:82-712).
    """

    def __init__(self, params, device=0):
        L = lib()
        h = ctypes.c_void_p()
        _check(L.fheacc_create(ctypes.byref(params), device, ctypes.byref(h)))
        self._h = h
        self.params = Params()
        _check(L.fheacc_get_params(h, ctypes.byref(self.params)), h)

    def close(self):
        if getattr(self, "_h", None):
            lib().fheacc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def last_error(self):
        return lib().fheacc_last_error(self._h).decode()

    def device_bytes(self):
        return lib().fheacc_device_bytes(self._h)

    def check(self, rc):
        _check(rc, self._h)

    def upload_bootstrap_key(self, btkey):
        """dma_write_bootstrap_key (myfpga.cpp:596-656)."""
        btkey = np.ascontiguousarray(btkey, dtype=np.uint64)
        self.check(lib().fheacc_upload_bootstrap_key(self._h, _p64(btkey), btkey.size))

    def upload_keyswitch_key(self, kskey):
        kskey = np.ascontiguousarray(kskey, dtype=np.uint64)
        self.check(lib().fheacc_upload_lwe_ks_key(self._h, _p64(kskey), kskey.size))

    def upload_subs_key(self, subs):
        """dma_write_subs_key (myfpga.cpp:658-712)."""
        subs = np.ascontiguousarray(subs, dtype=np.uint64)
        self.check(lib().fheacc_upload_subs_key(self._h, _p64(subs), subs.size))

    def verify_bootstrap_key(self, btkey):
        """dma_read_compare_bootstrap_key (myfpga.cpp:772-851): True if the
        device copy is what uploading btkey makes, False if it differs."""
        btkey = np.ascontiguousarray(btkey, dtype=np.uint64)
        rc = lib().fheacc_verify_bootstrap_key(self._h, _p64(btkey), btkey.size)
        if rc == EMISMATCH:
            return False
        self.check(rc)
        return True

    def verify_subs_key(self, subs):
        """dma_read_compare_subs_key (myfpga.cpp:853-925), as verify_bootstrap_key."""
        subs = np.ascontiguousarray(subs, dtype=np.uint64)
        rc = lib().fheacc_verify_subs_key(self._h, _p64(subs), subs.size)
        if rc == EMISMATCH:
            return False
        self.check(rc)
        return True

    def eval_bootstrap_batch(self, c1, c2, gates, flags=0):
        """eval_bootstrap (RLWE.cpp:726-786) of every (c1[i], c2[i], gates[i]),
        host arrays in, host array out."""
        w = self.params.n + 1
        c1 = np.ascontiguousarray(c1, dtype=np.uint64).reshape(-1, w)
        c2 = np.ascontiguousarray(c2, dtype=np.uint64).reshape(-1, w)
        g = np.ascontiguousarray(np.asarray(gates, dtype=np.int32).reshape(-1))
        if g.size == 1 and c1.shape[0] > 1:
            g = np.full(c1.shape[0], g[0], dtype=np.int32)
        out = np.zeros_like(c1)
        self.check(lib().fheacc_bootstrap(self._h, _p64(c1), _p64(c2), g.ctypes.data_as(_i32p), c1.shape[0],
                                          _p64(out), flags))
        return out

    def eval_bootstrap(self, c1, c2, gate, flags=0):
        """RLWE::eval_bootstrap (RLWE.cpp:726) of one gate."""
        return self.eval_bootstrap_batch(c1, c2, [gate], flags)[0]

    def _fixed(self, width, c1, c2, gates, flags):
        # fpga_eval_bootstrap_x* check the batch size of c1 and c2
        # (myfpga.cpp:1140-1144; x16 takes exactly 10, myfpga.cpp:1540-1544)
        if len(c1) != width or len(c2) != width or len(gates) != width:
            return None, -1
        try:
            return list(self.eval_bootstrap_batch(np.array(c1), np.array(c2), gates, flags)), 0
        except FheaccError as e:
            return None, e.code

    # The fixed-width calls give the CPU path's results (flags 0, the
    # bit-exact target) unless the caller asks for an FPGA issue order:
    # FLAG_FPGA_X1 for x1's (myfpga.cpp:1037-1046), FLAG_FPGA_COMPAT for
    # x4..x16's (myfpga.cpp:1200-1210).
    def gpu_eval_bootstrap_x1(self, c1, c2, gate, flags=0):
        """Counterpart of fpga_eval_bootstrap_x1 (myfpga.h:287): (result, rc)."""
        try:
            return self.eval_bootstrap(c1, c2, gate, flags), 0
        except FheaccError as e:
            return None, e.code

    def gpu_eval_bootstrap_x4(self, c1, c2, gates, flags=0):
        return self._fixed(4, c1, c2, gates, flags)

    def gpu_eval_bootstrap_x8(self, c1, c2, gates, flags=0):
        return self._fixed(8, c1, c2, gates, flags)

    def gpu_eval_bootstrap_x12(self, c1, c2, gates, flags=0):
        return self._fixed(12, c1, c2, gates, flags)

    def gpu_eval_bootstrap_x16(self, c1, c2, gates, flags=0):
        """fpga_eval_bootstrap_x16 takes exactly 10 gates (myfpga.cpp:1540-1544)."""
        return self._fixed(10, c1, c2, gates, flags)

    # device-pointer entry points (ints are raw device addresses, e.g.
    # torch.Tensor.data_ptr(); stream is a raw cudaStream_t or 0)
    def bootstrap_async(self, d_c1, d_c2, d_gates, count, d_out, flags=0, stream=0):
        self.check(lib().fheacc_bootstrap_async(self._h, d_c1, d_c2, d_gates, count, d_out, flags, stream or None))

    def bootstrap_noalloc(self, d_c1, d_c2, d_gates, count, d_out, flags=0, stream=0):
        """fheacc_bootstrap_noalloc: the same gate bootstraps with no device
        allocation (for callers that may not allocate), at most NOALLOC_MAX_GATES
        gates per call; the library's one scratch array is shared by all calls."""
        self.check(lib().fheacc_bootstrap_noalloc(self._h, d_c1, d_c2, d_gates, count, d_out, flags,
                                                  stream or None))

    def bootstrap_plain_async(self, d_c1, d_c2, d_gates, count, d_out, flags=0, stream=0):
        self.check(lib().fheacc_bootstrap_plain_async(self._h, d_c1, d_c2, d_gates, count, d_out, flags,
                                                      stream or None))

    def ntt_forward(self, d_polys, count, stream=0):
        self.check(lib().fheacc_ntt_forward(self._h, d_polys, count, stream or None))

    def ntt_inverse(self, d_polys, count, stream=0):
        self.check(lib().fheacc_ntt_inverse(self._h, d_polys, count, stream or None))

    def rlwe_mult_rgsw(self, d_acc, d_rgsw, d_out, count, stream=0):
        self.check(lib().fheacc_rlwe_mult_rgsw(self._h, d_acc, d_rgsw, d_out, count, stream or None))

    def blind_rotate_async(self, d_c1, d_c2, d_gates, count, d_acc, flags=0, stream=0):
        self.check(lib().fheacc_blind_rotate_async(self._h, d_c1, d_c2, d_gates, count, d_acc, flags, stream or None))

    def lwe_keyswitch_async(self, d_rlwe, count, d_out, stream=0):
        self.check(lib().fheacc_lwe_keyswitch_async(self._h, d_rlwe, count, d_out, stream or None))

    def lwe_modswitch_async(self, d_in, count, d_out, stream=0):
        self.check(lib().fheacc_lwe_modswitch_async(self._h, d_in, count, d_out, stream or None))

    def rlwe_substitute_async(self, d_in, count, f, d_out, stream=0):
        """RLWE_substitute (RLWE.cpp:444) of count NTT RLWEs."""
        self.check(lib().fheacc_rlwe_substitute_async(self._h, d_in, count, f, d_out, stream or None))

    def rlwe_keyswitch_async(self, d_in, count, d_ksk, d_out, stream=0):
        """RLWE_keyswitch (RLWE.cpp:464) with one key [digitKS_R][2][N]."""
        self.check(lib().fheacc_rlwe_keyswitch_async(self._h, d_in, count, d_ksk, d_out, stream or None))

    def subs_keyswitch_async(self, d_in, count, f, d_out, stream=0):
        """RLWE_keyswitch(RLWE_substitute(c, f), subs_key[f]) -- the RLWESUBS op."""
        self.check(lib().fheacc_subs_keyswitch_async(self._h, d_in, count, f, d_out, stream or None))

    def expand_RLWE(self, d_in, d_out, stream=0):
        """application::expand_RLWE (app.cpp:26): d_out = [N][2N] RLWEs."""
        self.check(lib().fheacc_expand_rlwe(self._h, d_in, d_out, stream or None))

    def CMUX(self, d_c0, d_c1, d_sel, d_out, count, in_stride=0, sel_shared=True, stream=0):
        """RLWE::CMUX (RLWE.cpp:788) of count pairs (fheacc_cmux_async)."""
        self.check(lib().fheacc_cmux_async(self._h, d_c0, d_c1, in_stride, d_sel, 1 if sel_shared else 0, d_out,
                                           count, stream or None))

    def blind_rotate_RLWE(self, d_in, d_rgsws, forward, d_out, count=1, stream=0):
        """RLWE::blind_rotate (RLWE.cpp:824): log2 N CMUXes with rotations."""
        self.check(lib().fheacc_rlwe_blind_rotate_async(self._h, d_in, d_rgsws, 1 if forward else 0, d_out, count,
                                                        stream or None))

    def homo_expand(self, d_packed, d_enc_sec, d_out, stream=0):
        """application::homo_expand (app.cpp:78): digitG RLWEs -> N RGSWs."""
        self.check(lib().fheacc_homo_expand(self._h, d_packed, d_enc_sec, d_out, stream or None))

    def sync(self, timeout_ms=0):
        self.check(lib().fheacc_sync(self._h, timeout_ms))

    def device_status(self):
        """Status bits of the context's finished device work (read and cleared);
        raises FheaccError when a kernel flagged its results invalid."""
        bits = ctypes.c_uint32()
        self.check(lib().fheacc_device_status(self._h, ctypes.byref(bits)))
        return bits.value

    def set_option(self, option, value):
        self.check(lib().fheacc_set_option(self._h, option, value))

    def kernel_launches(self):
        """Kernels this context has launched so far (one per kernel captured
        into a graph, at capture)."""
        n = ctypes.c_uint64()
        self.check(lib().fheacc_kernel_launches(self._h, ctypes.byref(n)))
        return n.value

    def kernel_times(self):
        """(blind rotation ms, key switch ms) of the last FLAG_PROFILE call."""
        ms = (ctypes.c_float * 2)()
        self.check(lib().fheacc_kernel_times(self._h, ms))
        return float(ms[0]), float(ms[1])

    def measure_imad_rate(self):
        """IMAD lane operations per second of this device."""
        v = ctypes.c_double()
        self.check(lib().fheacc_measure_imad_rate(self._h, ctypes.byref(v)))
        return v.value

    def measure_l2_read_rate(self):
        """L2 read bytes per second of this device (streaming probe)."""
        v = ctypes.c_double()
        self.check(lib().fheacc_measure_l2_read_rate(self._h, ctypes.byref(v)))
        return v.value

    def measure_components(self):
        """SM ns per unit of the blind-rotation step's pieces run alone:
        dict(ntt_fwd, ntt_digit, intt, mac) (fheacc_measure_components)."""
        v = (ctypes.c_double * 4)()
        self.check(lib().fheacc_measure_components(self._h, v))
        return dict(ntt_fwd=v[0], ntt_digit=v[1], intt=v[2], mac=v[3])

    def autotune(self, count, max_trials=64):
        """Times the blind rotation's launch options on a synthetic batch of
        `count` gates and keeps the fastest (fheacc_autotune). Returns the
        trials as dicts (regs_for_3, ctas_per_sm, group, ms)."""
        arr = (TuneTrial * max_trials)()
        n = ctypes.c_int()
        self.check(lib().fheacc_autotune(self._h, count, arr, max_trials, ctypes.byref(n)))
        return [{k: getattr(arr[i], k) for k, _ in TuneTrial._fields_} for i in range(min(n.value, max_trials))]


class Graph:
    """Batched bootstraps over one or more contexts replayed with one CUDA-graph
    launch (fheacc_graph_*). add() takes device pointers (ints) that must stay
    valid while the graph is used."""

    def __init__(self, concurrent=False):
        h = ctypes.c_void_p()
        _check(lib().fheacc_graph_create(ctypes.byref(h), GRAPH_CONCURRENT if concurrent else 0))
        self._h = h
        self._ctxs = []

    def _check(self, rc):
        if rc != OK:
            raise FheaccError(rc, (lib().fheacc_graph_last_error(self._h) or b"").decode())

    def add(self, ctx, d_c1, d_c2, d_gates, count, d_out):
        self._check(lib().fheacc_graph_add_bootstrap(self._h, ctx.handle, d_c1, d_c2, d_gates, count, d_out))
        self._ctxs.append(ctx)

    def launch(self, stream=0):
        self._check(lib().fheacc_graph_launch(self._h, stream or None))

    @property
    def batches(self):
        return lib().fheacc_graph_batches(self._h)

    def close(self):
        if getattr(self, "_h", None):
            lib().fheacc_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ serving
class Server:
    """Continuous-batching request loop (fheacc_server_*): requests are gate
    circuits over LWE ciphertexts; the ready gates of all admitted requests run
    in batched launches, up to two rounds in flight; admission by free room in
    a device pool (pool_ciphertexts=0: sized from the free device memory)."""

    def __init__(self, ctx, max_batch=4096, pool_ciphertexts=0):
        h = ctypes.c_void_p()
        ctx.check(lib().fheacc_server_create(ctx.handle, max_batch, pool_ciphertexts, ctypes.byref(h)))
        self._h = h
        self.ctx = ctx
        self.W = ctx.params.n + 1
        self._pending = {}

    def submit(self, inputs, gate_types, in1, in2, num_outputs):
        """Returns (request id, output array filled when the request completes)."""
        inputs = np.ascontiguousarray(inputs, dtype=np.uint64).reshape(-1, self.W)
        gt = np.ascontiguousarray(gate_types, dtype=np.int32)
        a = np.ascontiguousarray(in1, dtype=np.uint32)
        b = np.ascontiguousarray(in2, dtype=np.uint32)
        out = np.zeros((num_outputs, self.W), dtype=np.uint64)
        rid = ctypes.c_uint64()
        self.ctx.check(lib().fheacc_server_submit(self._h, _p64(inputs), inputs.shape[0], gt.ctypes.data_as(_i32p),
                                                  a.ctypes.data_as(_u32p), b.ctypes.data_as(_u32p), gt.size,
                                                  num_outputs, _p64(out), ctypes.byref(rid)))
        self._pending[rid.value] = (out, inputs, gt, a, b)   # keep buffers alive until done
        return rid.value, out

    def poll(self, max_done=256, timeout_ms=0):
        """[(request id, status, queue ms, latency ms, output array)]"""
        arr = (RequestDone * max_done)()
        n = ctypes.c_size_t()
        self.ctx.check(lib().fheacc_server_poll(self._h, arr, max_done, ctypes.byref(n), timeout_ms))
        res = []
        for i in range(n.value):
            d = arr[i]
            out = self._pending.pop(d.request_id)[0]
            res.append((d.request_id, d.status, d.queue_ms, d.latency_ms, out))
        return res

    def stats(self):
        st = ServerStats()
        self.ctx.check(lib().fheacc_server_stats(self._h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def close(self):
        if getattr(self, "_h", None):
            lib().fheacc_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def psi_equality_circuit(num_items, bits=32, or_reduce=False):
    """Gate circuit of a PSI-style equality query: the client item's `bits`
    encrypted bits (nodes 0..bits-1) against `num_items` encrypted server items
    (nodes bits + j*bits + b): per item `bits` XNOR gates and an AND tree; the
    item results are the last nodes (or one OR over them with or_reduce).
    Returns (gate_types, in1, in2, num_outputs)."""
    types, in1, in2 = [], [], []
    n_in = bits * (1 + num_items)
    roots_src = []

    def add(t, a, b):
        types.append(t)
        in1.append(a)
        in2.append(b)
        return n_in + len(types) - 1

    pending_roots = []
    for j in range(num_items):
        level = [add(XNOR, b, bits + j * bits + b) for b in range(bits)]
        while len(level) > 2:
            nxt = [add(AND, level[i], level[i + 1]) for i in range(0, len(level) - 1, 2)]
            if len(level) % 2:
                nxt.append(level[-1])
            level = nxt
        pending_roots.append(level)
    if bits == 1:
        raise ValueError("bits must be at least 2")
    roots = [add(AND, lv[0], lv[1]) for lv in pending_roots]   # one root per item, last
    if not or_reduce:
        return types, in1, in2, num_items
    level = roots
    while len(level) > 1:
        nxt = [add(OR, level[i], level[i + 1]) for i in range(0, len(level) - 1, 2)]
        if len(level) % 2:
            nxt.append(level[-1])
        level = nxt
    return types, in1, in2, 1
