"""Extracts the reference's golden transcripts into compact fixtures.

Sources (reference project: the path given as the first argument, else the
link oracle/_ref/reference that oracle/build_ref.sh leaves where it is mounted):
  cl_fhe_acc/verif/tests/mem_init_content/top_verify/bootstrap/bk/RLWExRGSW_output.txt
      one RLWE_mult_RGSW at N=1024, Q=0x7FFF801, BG=2^9, digitG=3
      (printed by the commented-out trace in FHE_ACC_runtime/src/RLWE.cpp:649-700)
  cl_fhe_acc/verif/tests/mem_init_content/top_verify/rlwesubs/bk/RLWESUBS_output.txt
      one RLWE_substitute(f=0) + RLWE_keyswitch at N=2048, Q=0x3FFFFFFFFED001
      (trace in FHE_ACC_runtime/src/app.cpp:37-68 and RLWE.cpp:481-504)
  cl_fhe_acc/verif/tests/mem_init_content/bk/param_{1k,2k}.txt

Writes rlwe_x_rgsw_1k.npz, rlwesubs_2k.npz and params.json next to this file.
Run:  python tests/golden/make_golden.py [REFERENCE_ROOT]
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
HEX = re.compile(r"^[0-9A-F]+$")


def blocks(path):
    """List of (header, [values]) for every header line followed by hex lines."""
    out = []
    cur = None
    with open(path) as f:
        for line in f:
            s = line.strip()
            if HEX.match(s):
                if cur is not None:
                    cur[1].append(int(s, 16))
            else:
                cur = (s, [])
                out.append(cur)
    return [(h, v) for h, v in out if v]


def rlwe_x_rgsw(ref):
    path = os.path.join(ref, "cl_fhe_acc/verif/tests/mem_init_content/top_verify/bootstrap/bk/RLWExRGSW_output.txt")
    bl = blocks(path)
    N = 1024
    for h, v in bl:
        assert len(v) == N, (h, len(v))
    hdr = [h for h, _ in bl]
    val = [np.array(v, dtype=np.uint64) for _, v in bl]
    i = 0
    acc = np.concatenate([val[0], val[1]])            # input RLWE content: poly a, poly b
    acc_time = np.concatenate([val[2], val[3]])       # time domain
    i = 4
    dG = 3
    # RGSW printed as "RLWE h, g": for g in 0..1, for h in 0..2 -> rows c_text[h][g]
    rgsw = np.zeros((dG, 2, 2, N), dtype=np.uint64)
    for g in range(2):
        for h in range(dG):
            rgsw[h, g, 0] = val[i]
            rgsw[h, g, 1] = val[i + 1]
            i += 2
    # loop a (g=0) then loop b (g=1): decomposed digit, RGSW a, RGSW b, tmp acc a, tmp acc b
    dec = np.zeros((dG, 2, N), dtype=np.uint64)
    partial = np.zeros((2, dG, 2, N), dtype=np.uint64)
    for g in range(2):
        for h in range(dG):
            dec[h, g] = val[i]
            assert np.array_equal(val[i + 1], rgsw[h, g, 0]) and np.array_equal(val[i + 2], rgsw[h, g, 1])
            partial[g, h, 0] = val[i + 3]
            partial[g, h, 1] = val[i + 4]
            i += 5
    out = np.concatenate([val[i], val[i + 1]])
    assert hdr[i].startswith("RLWE poly a") and i + 2 == len(val)
    np.savez_compressed(os.path.join(HERE, "rlwe_x_rgsw_1k.npz"), acc=acc, acc_time=acc_time, rgsw=rgsw,
                        dec=dec, out=out, Q=np.uint64(0x7FFF801), N=np.int64(N), BGbits=np.int64(9),
                        digitG=np.int64(dG), Q8=np.uint64(16776961), negQ8=np.uint64(117438720))


def rlwesubs(ref):
    path = os.path.join(ref, "cl_fhe_acc/verif/tests/mem_init_content/top_verify/rlwesubs/bk/RLWESUBS_output.txt")
    bl = blocks(path)
    N = 2048
    val = []
    for h, v in bl:
        assert len(v) == N, (h, len(v))
        val.append(np.array(v, dtype=np.uint64))
    L = 6
    ksk = np.zeros((L, 2, N), dtype=np.uint64)
    i = 0
    for k in range(L):
        ksk[k, 0] = val[i]
        ksk[k, 1] = val[i + 1]
        i += 2
    inp = np.concatenate([val[i], val[i + 1]]); i += 2
    inp_time = np.concatenate([val[i], val[i + 1]]); i += 2
    subs = np.concatenate([val[i], val[i + 1]]); i += 2
    dec = np.zeros((L, N), dtype=np.uint64)
    for k in range(L):
        dec[k] = val[i]
        i += 5   # decomposed a, multed a, multed b, acced a, acced b
    out = np.concatenate([val[i], val[i + 1]])
    assert i + 2 == len(val)
    np.savez_compressed(os.path.join(HERE, "rlwesubs_2k.npz"), ksk=ksk, inp=inp, inp_time=inp_time, subs=subs,
                        dec=dec, out=out, Q=np.uint64(18014398509404161), N=np.int64(N), Bks_R_bits=np.int64(9),
                        digitKS_R=np.int64(L), sub_factor=np.int64(0))


def params(ref):
    res = {}
    for tag in ("1k", "2k"):
        path = os.path.join(ref, "cl_fhe_acc/verif/tests/mem_init_content/bk/param_%s.txt" % tag)
        d = {}
        with open(path) as f:
            for line in f:
                m = re.match(r"^\s*(\w+)\s*=\s*([0-9A-Fa-f]+)", line)
                if m:
                    key, v = m.group(1), m.group(2)
                    d[key] = int(v, 10) if key == "k" else int(v, 16)
        res[tag] = {"Q": d["Q"], "iN": d["iN"], "ROU": d["ROU"], "k": d["k"]}
    with open(os.path.join(HERE, "params.json"), "w") as f:
        json.dump(res, f, indent=1)


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    ref = sys.argv[1] if len(sys.argv) > 1 else os.path.join(here, "..", "..", "oracle", "_ref", "reference")
    rlwe_x_rgsw(ref)
    rlwesubs(ref)
    params(ref)


if __name__ == "__main__":
    main()
