"""Generate the golden fixtures in this directory from the REFERENCE itself.

Runs only where the reference checkout is present (it is not available on
the GPU host; the fixtures it writes are committed):

* the reference's own known answers, read from its test modules
  (tests/test_reference.py:10-20 KNOWN, tests/test_gpu_logic.py:42-44 EDGE,
  tests/test_cuda_gpu.py:24-27 edge strings, tests/test_lib.py:62-69
  saturation) and evaluated by its ground truth (bench/reference.py:16-67);
* seeded random pairs / query-choice matrices evaluated by the reference's
  bitlev CPU API (bitlev/__init__.py:53-101, compiled from its sources into
  oracle/_ref by oracle/build_oracle.py) for every max_dist and dtype case;
* subsamples of the five benchmark workloads, evaluated the same way.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import importlib.util
import json
import os
import random
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import build_oracle  # noqa: E402
from editdist_bench_gb300 import workloads as W  # noqa: E402

REF = build_oracle.REF_SRC


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _b(s) -> str:
    """JSON-safe latin-1 text of str/bytes."""
    return s.decode("latin-1") if isinstance(s, (bytes, bytearray)) else s


def known_answers(bitlev, refmod):
    sys.path.insert(0, REF)              # the reference's tests import bench.*
    t_ref = _load("ref_test_reference", os.path.join(REF, "tests", "test_reference.py"))
    t_logic = _load("ref_test_gpu_logic", os.path.join(REF, "tests", "test_gpu_logic.py"))
    cases = []
    for a, b, d in t_ref.KNOWN:
        cases.append({"a": a, "b": b, "d": d, "src": "tests/test_reference.py:10-20"})
    for a, b in t_logic.EDGE:
        cases.append({"a": _b(a), "b": _b(b), "d": refmod.dp_distance(_b(a), _b(b)),
                      "src": "tests/test_gpu_logic.py:42-44"})
    A = ["", "", "abc", "a", "kitten", "\x00", "\xff" * 16, "".join(map(chr, range(256))), "x" * 300]
    B = ["", "abc", "", "b", "sitting", "\x00\x00", "\xff" * 15 + "\x00",
         "".join(map(chr, range(255, -1, -1))), "y" * 290]
    for a, b in zip(A, B):
        cases.append({"a": a, "b": b, "d": refmod.myers_distance(a, b),
                      "src": "tests/test_cuda_gpu.py:24-27"})
    # max_dist examples (tests/test_lib.py:30-34) and every KNOWN pair under a few k
    thresholded = [{"a": "kitten", "b": "sitting", "k": 1, "d": bitlev.distance("kitten", "sitting", max_dist=1),
                    "src": "tests/test_lib.py:34"}]
    for c in cases:
        for k in (0, 1, 2, 5):
            thresholded.append({"a": c["a"], "b": c["b"], "k": k,
                                "d": int(bitlev.pairwise([c["a"]], [c["b"]], max_dist=k)[0]),
                                "src": c["src"] + " (bitlev.pairwise max_dist)"})
    # dtype saturation (tests/test_lib.py:62-69; tests/test_gpu_logic.py:121-122)
    Q, C = ["a" * 300, "b"], ["c" * 10, "b" * 400]
    sat = {"Q": Q, "C": C, "int32": bitlev.cdist(Q, C).tolist(),
           "uint8": bitlev.cdist(Q, C, dtype="uint8").tolist(),
           "uint16": bitlev.cdist(Q, C, dtype=np.uint16).tolist(),
           "pair_x300_empty_uint8": int(bitlev.pairwise(["x" * 300], [""], dtype=np.uint8)[0]),
           "store8": {"in": [0, 7, 254, 255, 256, 9999], "out": [0, 7, 254, 255, 255, 255]},
           "src": "tests/test_lib.py:62-69, tests/test_gpu_logic.py:121-122"}
    return {"exact": cases, "thresholded": thresholded, "saturation": sat}


def _rand_pairs(seed, n):
    rng = random.Random(seed)
    A, B = [], []
    alphas = [b"AB", b"ACGT", b"ACGT\x00", b"abcdefghijklmnopqrstuvwxyz ", b"\x00\x01\xff",
              bytes(range(256))]
    lengths = [0, 1, 2, 3, 4, 5, 7, 15, 16, 17, 31, 32, 33, 63, 64, 65, 100, 127, 128, 129,
               191, 192, 193, 255, 256, 257, 300, 511, 512, 513, 600, 1000]
    for _ in range(n):
        al = rng.choice(alphas)
        L = rng.choice(lengths) if rng.random() < 0.6 else rng.randrange(0, 700)
        a = bytearray(rng.choice(al) for _ in range(L))
        kind = rng.randrange(4)
        if kind == 0:
            b = bytearray(rng.choice(al) for _ in range(rng.randrange(0, L + 40)))
        elif kind == 1:   # few edits: long common prefix/suffix
            b = bytearray(a)
            for _ in range(rng.randrange(0, 12)):
                i = rng.randrange(len(b) + 1)
                op = rng.randrange(3)
                if op == 0 and i < len(b): b[i] = rng.choice(al)
                elif op == 1: b.insert(i, rng.choice(al))
                elif i < len(b): del b[i]
        elif kind == 2:   # prefix / suffix of a
            b = a[: rng.randint(0, L)] if rng.random() < 0.5 else a[rng.randint(0, L):]
        else:
            b = bytearray(a)
        if rng.random() < 0.5:
            a, b = b, a
        A.append(bytes(a))
        B.append(bytes(b))
    return A, B


def random_suite(bitlev):
    A, B = _rand_pairs(20261203, 1500)
    pa, pb = oracle.pack(A), oracle.pack(B)
    out = {"a_buf": pa[0], "a_off": pa[1], "b_buf": pb[0], "b_off": pb[1]}
    for k in (None, 0, 1, 2, 3, 5, 8, 17, 100):
        tag = "none" if k is None else str(k)
        out[f"pairs_k{tag}_int32"] = bitlev.pairwise(A, B, max_dist=k)
        if k in (None, 3, 100):
            out[f"pairs_k{tag}_uint8"] = bitlev.pairwise(A, B, max_dist=k, dtype=np.uint8)
            out[f"pairs_k{tag}_uint16"] = bitlev.pairwise(A, B, max_dist=k, dtype=np.uint16)
    Qs, Cs = _rand_pairs(7, 60)
    Q = Qs[:30] + [b"", b"a" * 64, b"b" * 65, b"c" * 512, b"d" * 513, b"e" * 1000, b"q" * 600]
    C = Cs[:80] + [b"", b"aaa", b"b" * 70, b"c" * 500, b"xyz"]
    pq, pc = oracle.pack(Q), oracle.pack(C)
    out.update({"q_buf": pq[0], "q_off": pq[1], "c_buf": pc[0], "c_off": pc[1]})
    for k in (None, 0, 2, 15):
        tag = "none" if k is None else str(k)
        out[f"cross_k{tag}_int32"] = bitlev.cdist(Q, C, max_dist=k)
        out[f"cross_k{tag}_uint8"] = bitlev.cdist(Q, C, max_dist=k, dtype=np.uint8)
    out["cross_knone_uint16"] = bitlev.cdist(Q, C, dtype=np.uint16)
    return out


def config_suite(bitlev):
    out = {}
    w1 = W.config1(n=4096)
    w3 = W.config3(n=4096)
    for tag, w in (("c1", w1), ("c3", w3)):
        A, B = W.unpack(w.a), W.unpack(w.b)
        out[f"{tag}_a_buf"], out[f"{tag}_a_off"] = w.a
        out[f"{tag}_b_buf"], out[f"{tag}_b_off"] = w.b
        out[f"{tag}_out"] = bitlev.pairwise(A, B, max_dist=w.max_dist, dtype=w.dtype)
    # reference.py (DP) on a subsample of config 1, as the configuration asks
    refmod = _load("ref_reference", os.path.join(REF, "bench", "reference.py"))
    A, B = W.unpack(W.take(w1.a, np.arange(300))), W.unpack(W.take(w1.b, np.arange(300)))
    out["c1_dp300"] = np.array([refmod.dp_distance(a.decode(), b.decode()) for a, b in zip(A, B)],
                               dtype=np.int32)
    w2 = W.config2(nq=48, nc=1024)
    w4 = W.config4(nq=24, nc=1024)
    for tag, w, ks in (("c2", w2, ((None, "int32"), (2, "uint8"))), ("c4", w4, ((4, "uint8"),))):
        Q, C = W.unpack(w.q), W.unpack(w.c)
        out[f"{tag}_q_buf"], out[f"{tag}_q_off"] = w.q
        out[f"{tag}_c_buf"], out[f"{tag}_c_off"] = w.c
        for k, dt in ks:
            out[f"{tag}_k{'none' if k is None else k}_{dt}"] = bitlev.cdist(Q, C, max_dist=k, dtype=dt)
    probs = W.config5(n_problems=6, scale=1 / 256)
    for i, p in enumerate(probs):
        Q, C = W.unpack(p.q), W.unpack(p.c)
        out[f"c5_{i}_q_buf"], out[f"c5_{i}_q_off"] = p.q
        out[f"c5_{i}_c_buf"], out[f"c5_{i}_c_off"] = p.c
        out[f"c5_{i}_k"] = np.array([p.max_dist])
        out[f"c5_{i}_dtype"] = np.array([p.dtype])
        out[f"c5_{i}_out"] = bitlev.cdist(Q, C, max_dist=p.max_dist, dtype=p.dtype)
    return out


def main():
    build_oracle.build_ref()
    bitlev = oracle.ref_bitlev()
    refmod = _load("ref_reference", os.path.join(REF, "bench", "reference.py"))
    with open(os.path.join(HERE, "known.json"), "w") as f:
        json.dump(known_answers(bitlev, refmod), f, indent=0)
    np.savez_compressed(os.path.join(HERE, "random_suite.npz"), **random_suite(bitlev))
    np.savez_compressed(os.path.join(HERE, "configs.npz"), **config_suite(bitlev))
    for f in sorted(os.listdir(HERE)):
        print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
