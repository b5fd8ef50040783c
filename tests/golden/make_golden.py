"""Generates the golden fixtures in tests/golden/ from the REFERENCE itself.

Run here (where the reference sources are mounted) after building the
reference tools with ``sh oracle/ref/build_ref.sh``; the fixtures are then
committed and the tests read only them (the reference does not exist where
the GPU tests run).

Fixtures:
  ref_<spot>.npz      every integer artifact of the reference compiler
                      (cuda/gpu_cfr.cu:1331-1827) for small spots
  ref_hashes.json     sha256 per artifact for the large spots
  tiny_check.json     known-answer EVs printed by tools/tiny_check.cpp
  eval_keys.npz       reference strength keys of seeded 7-card hands
  bet_actions.json    reference pf::betActions on seeded betting states
  ranges.json         reference parseRange weights for range strings
  api_routes.json     (method, path) of every route of the reference's HTTP
                      API (python/pps_api.py), read from its source as text
  ref_treebuf.json    byte offset of every TreeBuf member (the argument
                      block of the reference kernels, cuda/gpu_cfr.cu:
                      132-201) and its size, as compiled from the source
  ref_solution_v1.pps a "PPS1" version-1 solution file written by the
                      reference's own save() (cuda/gpu_cfr.cu:2743-2785) for
                      a small river spot, rows set to a fixed pattern, with
                      ref_solution_v1.json (the spot, sizes, sha256)
"""
from __future__ import annotations

import hashlib
import json
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(REPO, "oracle", "_ref")
# The reference checkout: PPS_REFERENCE, else `reference` beside this repository.
REF_SRC = os.environ.get("PPS_REFERENCE") or os.path.join(os.path.dirname(REPO), "reference")
sys.path.insert(0, os.path.join(REPO, "cuda-poker-solver_gb300"))
from pps import workloads as wl  # noqa: E402

DT = {"i": np.int32, "q": np.int64, "B": np.uint8, "f": np.float32, "d": np.float64}


def read_dump(path):
    b = open(path, "rb").read()
    assert b[:8] == b"PPSDUMP1"
    n = struct.unpack_from("<I", b, 8)[0]
    o = 12
    out = {}
    for _ in range(n):
        ln = struct.unpack_from("<H", b, o)[0]
        o += 2
        name = b[o:o + ln].decode()
        o += ln
        t = chr(b[o])
        o += 1
        cnt = struct.unpack_from("<Q", b, o)[0]
        o += 8
        a = np.frombuffer(b, dtype=DT[t], count=cnt, offset=o).copy()
        o += a.nbytes
        out[name] = a
    return out


def range_arg(r, tmp, tag):
    if isinstance(r, str):
        return r
    path = os.path.join(tmp, tag + ".w")
    np.asarray(r, dtype="<f8").tofile(path)
    return "@" + path


def capture(spot: wl.Spot):
    assert spot.street_cfgs is None, "the reference has one config for all streets"
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "dump.bin")
        cmd = [os.path.join(REF_BIN, "ref_capture"), out, spot.board_text(),
               range_arg(spot.oop, tmp, "oop"), range_arg(spot.ip, tmp, "ip"),
               str(spot.pot), str(spot.stack), spot.cfg.bet_text(),
               spot.cfg.raise_text(), str(spot.cfg.max_raises)]
        subprocess.run(cmd, check=True)
        return read_dump(out)


def edge_spots():
    return [wl.turn_short(), wl.flop_short(), wl.river_geo(), wl.river_empty()]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_probe(mode, lines):
    p = subprocess.run([os.path.join(REF_BIN, "ref_probe"), mode],
                       input="\n".join(lines) + "\n", capture_output=True,
                       text=True, check=True)
    return p.stdout.strip("\n").split("\n")


def treebuf_layout():
    out = subprocess.run([os.path.join(REF_BIN, "ref_capture"), "--treebuf"],
                         capture_output=True, text=True, check=True).stdout
    members, size = [], None
    for line in out.split("\n"):
        f = line.split()
        if len(f) != 2:
            continue
        if f[0] == "sizeof":
            size = int(f[1])
        else:
            members.append([f[0], int(f[1])])
    json.dump({"members": members, "size": size},
              open(os.path.join(HERE, "ref_treebuf.json"), "w"), indent=0)


def api_routes():
    import re
    src = open(os.path.join(REF_SRC, "python", "pps_api.py")).read()
    routes = sorted({(m.upper(), p) for m, p, rest in
                     re.findall(r'@app\.(get|post|delete|put)\("([^"]+)"([^)]*)\)', src)
                     if "include_in_schema=False" not in rest})
    json.dump([list(r) for r in routes], open(os.path.join(HERE, "api_routes.json"), "w"),
              indent=0)


# The solution-file golden: a small river spot saved by the reference's own
# save() with rows set to ref_capture's fixed pattern.
SOLUTION_SPOT = {"board": "Qs9h2d7c5d", "oop": "TT+,AKo", "ip": "AQ+,KQs", "pot": 200,
                 "stack": 500, "bets": "0.75,a", "raises": "2.5,3", "max_raises": 0,
                 "iterations": 300}


def solution_file():
    sp = SOLUTION_SPOT
    path = os.path.join(HERE, "ref_solution_v1.pps")
    subprocess.run([os.path.join(REF_BIN, "ref_capture"), "--save", path, str(sp["iterations"]),
                    sp["board"], sp["oop"], sp["ip"], str(sp["pot"]), str(sp["stack"]),
                    sp["bets"], sp["raises"], str(sp["max_raises"])], check=True)
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "load.bin")
        subprocess.run([os.path.join(REF_BIN, "ref_capture"), "--load", path, out], check=True)
        d = read_dump(out)
    meta = dict(sp)
    meta.update({"num_nodes": int(d["numNodes"][0]), "reg_total": int(d["regTotal"][0]),
                 "sha256": hashlib.sha256(open(path, "rb").read()).hexdigest()})
    json.dump(meta, open(os.path.join(HERE, "ref_solution_v1.json"), "w"), indent=1)
    print("solution file", meta["num_nodes"], "nodes,", meta["reg_total"], "rows")


def main():
    if sys.argv[1:] == ["--api-routes"]:
        api_routes()
        return
    if sys.argv[1:] == ["--solution-file"]:
        solution_file()
        return
    if not os.path.exists(os.path.join(REF_BIN, "ref_capture")):
        raise SystemExit("build the reference tools first: sh oracle/ref/build_ref.sh")
    treebuf_layout()
    api_routes()
    if sys.argv[1:] == ["--treebuf"]:
        return
    small = [wl.river_c1(), wl.turn_api(), wl.turn_tiny()] + edge_spots()
    for spot in small:
        arrs = capture(spot)
        np.savez_compressed(os.path.join(HERE, "ref_%s.npz" % spot.name), **arrs)
        print(spot.name, int(arrs["numNodes"][0]), "nodes")
    hashes = {}
    for spot in [wl.turn_w52(), wl.turn_c3(), wl.turn_c2(uniform_config=True),
                 wl.flop_small()]:
        arrs = capture(spot)
        hashes[spot.name] = {k: [sha(v), int(v.size)] for k, v in arrs.items()}
        print(spot.name, int(arrs["numNodes"][0]), "nodes (hashed)")
    json.dump(hashes, open(os.path.join(HERE, "ref_hashes.json"), "w"), indent=0)

    tiny = {}
    out = subprocess.run([os.path.join(REF_BIN, "tiny_check")], capture_output=True,
                         text=True, check=True).stdout
    for line in out.splitlines():
        for tag in ("TINY", "M7", "M9"):
            if line.startswith(tag + ":"):
                f = line.split()
                tiny[tag] = {"ev0": float(f[2]), "ev1": float(f[4])}
    json.dump(tiny, open(os.path.join(HERE, "tiny_check.json"), "w"), indent=1)

    rng = wl.SplitMix64(7)
    hands = []
    for _ in range(20000):
        cards = []
        while len(cards) < 7:
            c = rng.next() % 52
            if c not in cards:
                cards.append(c)
        hands.append(cards)
    for _ in range(4000):  # a hole card repeating a board card (blocked combos)
        cards = []
        while len(cards) < 6:
            c = rng.next() % 52
            if c not in cards:
                cards.append(c)
        cards.insert(1, cards[2 + rng.next() % 4])
        hands.append(cards)
    keys = run_probe("eval", [" ".join(map(str, h)) for h in hands])
    np.savez_compressed(os.path.join(HERE, "eval_keys.npz"),
                        hands=np.array(hands, dtype=np.uint8),
                        keys=np.array([int(k) for k in keys], dtype=np.uint64))

    rng = wl.SplitMix64(11)
    states = []
    for _ in range(6000):
        pot = 1 + rng.next() % 600
        stack = rng.next() % 2000
        prev = rng.next() % (stack + 1) if rng.uniform() < 0.6 else 0
        mine = rng.next() % (prev + 1)
        actor = rng.next() % 2
        sc = (mine, prev) if actor == 0 else (prev, mine)
        if rng.uniform() < 0.5:
            sc = (sc[1], sc[0]) if rng.uniform() < 0.5 else sc
        nb = rng.next() % 5
        bets = sorted({[0.25, 0.33, 0.5, 0.75, 1.0, 1.25, 1.5, 2.0][rng.next() % 8]
                       for _ in range(nb)})
        nr = rng.next() % 3
        raises = sorted({[2.0, 2.5, 3.0, 4.0][rng.next() % 4] for _ in range(nr)})
        st = {"pot": pot, "stack": stack, "sc0": sc[0], "sc1": sc[1],
              "actor": actor, "after_allin": int(rng.uniform() < 0.2),
              "num_bets": rng.next() % 4, "num_streets": 1 + rng.next() % 3,
              "allin": int(rng.uniform() < 0.5), "geo": int(rng.uniform() < 0.2),
              "max_raises": rng.next() % 4,
              "add": [1.5, 0.0, 3.0][rng.next() % 3],
              "force": [0.15, 0.0, 0.3][rng.next() % 3],
              "merge": [0.1, 0.0, 0.25][rng.next() % 3],
              "bets": bets, "raises": raises}
        states.append(st)
    lines = []
    for s in states:
        lines.append(" ".join(str(x) for x in [
            s["pot"], s["stack"], s["sc0"], s["sc1"], s["actor"], s["after_allin"],
            s["num_bets"], s["num_streets"], s["allin"], s["geo"], s["max_raises"],
            repr(s["add"]), repr(s["force"]), repr(s["merge"]), len(s["bets"]),
            len(s["raises"])] + [repr(x) for x in s["bets"] + s["raises"]]))
    outs = run_probe("bet", lines)
    for s, o in zip(states, outs):
        f = [int(x) for x in o.split()]
        s["out"] = [[f[1 + 2 * i], f[2 + 2 * i]] for i in range(f[0])]
    json.dump(states, open(os.path.join(HERE, "bet_actions.json"), "w"))

    range_strs = ["AA", "AKs", "AKo", "AK", "TT+", "A9s+", "T9s+", "A5s-A2s",
                  "98s-65s", "55-22", "AA:0.5,KK", "AK,AA", "22+,A9s+,KTs+,QJs,JTs,T9s",
                  "22+,A9s+,KTs+,QJs,JTs,T9s,AQo+", "TT+,AKo", "AQ+,KQs", "99+",
                  "KTo-K7o", "KQo-JTo", " QQ , JJ:0.25 ", "AA,AA", "XX", "AKx", "A",
                  "22-55", "A2s-A5s", "AK-QJ", "AA-KK", "T9o+", "AJo+:0.3"]
    outs = run_probe("range", range_strs)
    ranges = {}
    for s, o in zip(range_strs, outs):
        ranges[s] = None if o == "ERR" else [float(x) for x in o.split()]
    json.dump(ranges, open(os.path.join(HERE, "ranges.json"), "w"))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
