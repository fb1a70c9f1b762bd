#!/usr/bin/env python3
"""Regenerates tests/golden/golden.json by running the reference's own CPU code.

oracle/_ref/ref_driver is compiled (``make -C oracle ref``) from the
reference's unmodified headers (dloghin/plonky3-gpu, src/include) plus
oracle/ref_driver.cpp, which parses arguments, draws seeded inputs in the
reference tests' convention (std::mt19937(seed), ``rng() % p``) and adapts the
reference's DuplexChallenger for TwoAdicFriPcs::open.  This
script runs it over a fixed list of cases and stores the outputs: small
arrays in full, large ones as a SHA-256 of their little-endian bytes plus the
leading values.  Needs the reference sources, so it runs only where they are
mounted; the committed JSON is what the tests read.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(REPO, "oracle", "_ref", "ref_driver")
FULL_LIMIT = 4096


def run(*args) -> bytes:
    with tempfile.NamedTemporaryFile(delete=False) as f:
        path = f.name
    try:
        subprocess.run([DRIVER, path, *[str(a) for a in args]], check=True)
        with open(path, "rb") as f:
            return f.read()
    finally:
        os.unlink(path)


def summarize(arr: np.ndarray) -> dict:
    arr = np.ascontiguousarray(arr)
    d = {"n": int(arr.size), "sha256": hashlib.sha256(arr.tobytes()).hexdigest()}
    if arr.size <= FULL_LIMIT:
        d["values"] = [int(x) for x in arr.reshape(-1)]
    else:
        d["head"] = [int(x) for x in arr.reshape(-1)[:64]]
    return d


def parse_layers(raw: bytes, dtype, digest: int):
    nl = int(np.frombuffer(raw[:8], np.uint64)[0])
    sizes = np.frombuffer(raw[8:8 + 8 * nl], np.uint64).astype(int).tolist()
    body = np.frombuffer(raw[8 + 8 * nl:], dtype)
    layers, off = [], 0
    for s in sizes:
        layers.append(body[off:off + s * digest].reshape(s, digest))
        off += s * digest
    return sizes, layers


def main() -> int:
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref"], check=True)
    g: dict = {"generator": "tests/golden/make_golden.py via oracle/_ref/ref_driver"}

    c = run("consts")
    bb = np.frombuffer(c[: 4 * (64 + 64 + 13)], np.uint32)
    gl = np.frombuffer(c[4 * (64 + 64 + 13):], np.uint64)
    g["consts"] = {
        "bb16_initial": bb[:64].tolist(), "bb16_terminal": bb[64:128].tolist(),
        "bb16_internal": bb[128:141].tolist(),
        "gl8_initial": [int(x) for x in gl[:32]], "gl8_terminal": [int(x) for x in gl[32:64]],
        "gl8_internal": [int(x) for x in gl[64:86]],
    }

    k = run("kat")
    ku = np.frombuffer(k[:4 * (1 + 1 + 4 + 28)], np.uint32)
    kg = np.frombuffer(k[4 * (1 + 1 + 4 + 28):], np.uint64)
    g["kat"] = {
        "bb_two_adic_27": int(ku[0]), "bb4_dth_root": int(ku[1]),
        "bb4_ext_two_adic_28": ku[2:6].tolist(), "bb_two_adic": ku[6:34].tolist(),
        "gl_two_adic": [int(x) for x in kg],
    }

    lde = []
    bb_cases = [(0, 3, 1, 11, 1), (1, 1, 1, 12, 1), (2, 5, 2, 13, 1), (3, 4, 1, 111, 1),
                (4, 3, 3, 222, 1), (5, 8, 2, 333, 1), (6, 1, 1, 444, 1), (7, 17, 1, 555, 1),
                (10, 8, 1, 777, 1), (9, 33, 2, 456, 1), (8, 64, 3, 123, 1), (6, 5, 1, 321, 0),
                (11, 24, 1, 99, 1), (12, 16, 1, 1, 1), (13, 5, 2, 5, 1), (14, 3, 1, 8, 1)]
    for (lh, w, lb, seed, br) in bb_cases:
        raw = np.frombuffer(run("lde", "bb", lh, w, lb, seed, 31, br), np.uint32)
        lde.append({"field": "bb", "log_h": lh, "w": w, "log_blowup": lb, "seed": seed,
                    "shift": 31, "bitrev": br, "out": summarize(raw)})
    gl_cases = [(0, 2, 2, 21, 1), (3, 4, 2, 22, 1), (5, 3, 1, 23, 1), (8, 8, 2, 24, 1),
                (10, 16, 2, 7, 1), (6, 2, 3, 25, 0)]
    for (lh, w, lb, seed, br) in gl_cases:
        raw = np.frombuffer(run("lde", "gl", lh, w, lb, seed, 7, br), np.uint64)
        lde.append({"field": "gl", "log_h": lh, "w": w, "log_blowup": lb, "seed": seed,
                    "shift": 7, "bitrev": br, "out": summarize(raw)})
    g["lde"] = lde

    dft = []
    for kind in ("dft", "idft", "coset_dft", "coset_idft"):
        for (lh, w, seed) in ((3, 2, 31), (6, 3, 32), (0, 2, 33)):
            raw = np.frombuffer(run("dft", "bb", kind, lh, w, seed, 31), np.uint32)
            dft.append({"kind": kind, "log_h": lh, "w": w, "seed": seed, "shift": 31,
                        "out": summarize(raw)})
    g["dft"] = dft

    perm = []
    for kind, n, seed, width, dt in (("bb16", 4, 5, 16, np.uint32), ("bb16zero", 2, 6, 16, np.uint32),
                                     ("bb16zero_generic", 2, 6, 16, np.uint32),
                                     ("gl8", 4, 7, 8, np.uint64)):
        raw = np.frombuffer(run("perm", kind, n, seed), dt).reshape(n, 2, width)
        perm.append({"kind": kind, "inputs": [[int(x) for x in r] for r in raw[:, 0]],
                     "outputs": [[int(x) for x in r] for r in raw[:, 1]]})
    g["perm"] = perm

    hashes = []
    for ln in (0, 1, 7, 8, 9, 15, 16, 17, 33, 256):
        raw = np.frombuffer(run("hash", "bb16", ln, 1000 + ln), np.uint32)
        hashes.append({"kind": "bb16", "len": ln, "seed": 1000 + ln, "digest": raw.tolist()})
    for ln in (0, 1, 3, 4, 5, 8, 13):
        raw = np.frombuffer(run("hash", "gl8", ln, 2000 + ln), np.uint64)
        hashes.append({"kind": "gl8", "len": ln, "seed": 2000 + ln, "digest": [int(x) for x in raw]})
    g["hash"] = hashes

    comp = []
    for kind, dt in (("bb16", np.uint32), ("gl8", np.uint64)):
        for seed in (1, 2):
            raw = np.frombuffer(run("compress", kind, seed), dt)
            comp.append({"kind": kind, "seed": seed, "digest": [int(x) for x in raw]})
    g["compress"] = comp

    mm = []
    shape_sets = [
        ("bb16", 0, 41, ["8x16"]), ("bb16", 0, 42, ["16x9", "8x4"]),
        ("bb16", 0, 43, ["32x3", "8x9", "32x2", "2x5"]),
        ("bb16", 0, 44, ["64x16", "16x8", "4x3", "1x2"]),
        ("bb16", 1, 45, ["16x3", "4x9", "16x2", "2x5", "1x4"]),
        ("bb16", 2, 46, ["32x8"]), ("bb16", 0, 47, ["8x24", "8x1"]), ("bb16", 0, 48, ["1x5"]),
        ("bb16", 0, 49, ["4x2", "128x7", "32x300", "128x1", "8x17"]),
        ("bb16zero", 0, 50, ["16x16", "8x8"]),
        ("gl8", 0, 51, ["16x4", "4x3", "16x5"]), ("gl8", 1, 52, ["8x8"]),
    ]
    for kind, cap, seed, shapes in shape_sets:
        dt, dg = (np.uint64, 4) if kind == "gl8" else (np.uint32, 8)
        sizes, layers = parse_layers(run("mmcs", kind, cap, seed, *shapes), dt, dg)
        mm.append({"kind": kind, "cap_height": cap, "seed": seed, "shapes": shapes, "sizes": sizes,
                   "layers": [[[int(x) for x in d] for d in l] for l in layers]})
    g["mmcs"] = mm

    cm = []
    for (h, w, seed) in ((8, 4, 61), (5, 3, 62), (1, 8, 63), (13, 16, 64), (64, 8, 65)):
        sizes, layers = parse_layers(run("commit_matrix", h, w, seed), np.uint32, 8)
        cm.append({"h": h, "w": w, "seed": seed, "sizes": sizes,
                   "layers": [[[int(x) for x in d] for d in l] for l in layers]})
    g["commit_matrix"] = cm

    commits = []
    for (lh, w, lb, seed, cap) in ((12, 16, 1, 1, 0), (6, 8, 1, 3, 0), (8, 20, 2, 4, 1)):
        sizes, layers = parse_layers(run("commit", lh, w, lb, seed, cap), np.uint32, 8)
        allb = np.concatenate([l.reshape(-1) for l in layers])
        commits.append({"log_h": lh, "w": w, "log_blowup": lb, "seed": seed, "cap_height": cap,
                        "shift": 31, "sizes": sizes, "cap": [[int(x) for x in d] for d in layers[-1]],
                        "layers_sha256": hashlib.sha256(allb.tobytes()).hexdigest()})
    g["commit"] = commits

    pcs = []
    for seed, shapes in ((3, ["5x16", "8x16", "7x16"]), (9, ["4x3", "4x5"]), (10, ["6x1"])):
        raw = np.frombuffer(run("pcs_commit", seed, *shapes), np.uint32)
        pcs.append({"seed": seed, "shapes": shapes, "log_blowup": 1, "shift": 1, "root": raw.tolist()})
    g["pcs_commit"] = pcs

    opens = []
    for seed, shapes in ((3, ["5x16", "8x16", "7x16"]), (11, ["6x5", "6x3"]), (12, ["9x2", "4x7"])):
        raw = np.frombuffer(run("pcs_open", seed, *shapes), np.uint32)
        n_open = sum(int(s.split("x")[1]) for s in shapes) * 4
        o = 8 + n_open
        rounds = int(raw[o])
        tail = o + 10
        commits = raw[tail + 8:tail + 8 + 8 * rounds].reshape(rounds, 8).tolist()
        nf = int(raw[tail + 8 + 8 * rounds])
        end = tail + 9 + 8 * rounds + 4 * nf
        final = raw[tail + 9 + 8 * rounds:end].reshape(nf, 4).tolist()
        pow_witness = int(raw[end]) | (int(raw[end + 1]) << 32)
        cur = [end + 2]

        def take(n):
            v = raw[cur[0]:cur[0] + n]
            cur[0] += n
            return v

        queries = []
        for _ in range(int(take(1)[0])):
            steps = []
            for _ in range(int(take(1)[0])):
                la = int(take(1)[0])
                ns = int(take(1)[0])
                sib = take(4 * ns).reshape(ns, 4).tolist()
                npf = int(take(1)[0])
                steps.append({"log_arity": la, "siblings": sib, "path": take(8 * npf).reshape(npf, 8).tolist()})
            queries.append(steps)
        assert cur[0] == raw.size, (cur[0], raw.size)
        opens.append({"seed": seed, "shapes": shapes, "log_blowup": 1, "shift": 1,
                      "fri": {"log_final_poly_len": 0, "max_log_arity": 1, "commit_pow_bits": 0,
                              "query_pow_bits": 8, "query_pow_witness": pow_witness},
                      "zeta": raw[0:4].tolist(), "alpha": raw[4:8].tolist(),
                      "opened": raw[8:o].tolist(), "fri_rounds": rounds,
                      "log_arity0": int(raw[o + 1]), "commit0": raw[o + 2:o + 10].tolist(),
                      "pcs_root": raw[tail:tail + 8].tolist(), "commits": commits, "final_poly": final,
                      "num_queries": 10, "query_openings": queries})
    g["pcs_open"] = opens

    grinds = []
    bits_list = [1, 8, 12, 0, 16]
    for seed, n_obs in ((1, 0), (2, 1), (3, 5), (4, 6), (5, 7), (6, 8), (7, 13), (8, 15)):
        raw = run("grind", seed, n_obs, *bits_list)
        ws, samples = [], []
        for i in range(len(bits_list)):
            chunk = raw[i * 12:(i + 1) * 12]
            ws.append(int(np.frombuffer(chunk[:8], np.uint64)[0]))
            samples.append(int(np.frombuffer(chunk[8:], np.uint32)[0]))
        grinds.append({"seed": seed, "n_obs": n_obs, "bits": bits_list, "witness": ws, "sample_after": samples})
    raw = run("grind", 9, 3, 20)
    grinds.append({"seed": 9, "n_obs": 3, "bits": [20],
                   "witness": [int(np.frombuffer(raw[:8], np.uint64)[0])],
                   "sample_after": [int(np.frombuffer(raw[8:12], np.uint32)[0])]})
    g["grind"] = grinds

    folds = []
    for (lh, la, seed, mode) in ((4, 1, 0xDEADBEEF, 0), (6, 1, 71, 0), (10, 1, 72, 0), (5, 2, 73, 0),
                                 (7, 2, 74, 0), (6, 3, 75, 0), (8, 3, 76, 0), (4, 1, 77, 1),
                                 (5, 2, 78, 1), (6, 3, 79, 1), (3, 3, 80, 0)):
        raw = np.frombuffer(run("fold", lh, la, seed, mode), np.uint32)
        folds.append({"log_height": lh, "log_arity": la, "seed": seed, "beta_mode": mode,
                      "beta": raw[:4].tolist(), "out": summarize(raw[4:])})
    g["fold"] = folds

    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(g, f, indent=None, separators=(",", ":"))
        f.write("\n")
    print("wrote", os.path.join(HERE, "golden.json"))
    return 0


if __name__ == "__main__":
    sys.exit(main())
