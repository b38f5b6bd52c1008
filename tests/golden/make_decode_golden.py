"""Regenerate tests/golden/decode.json from the REFERENCE library: error codes
and outputs of blst_p1_uncompress / blst_p1_deserialize / blst_p1_affine_in_g1
over seeded crafted encodings (valid points, infinity encodings, flag errors,
non-canonical coordinates, off-curve and on-curve non-subgroup points, the
(0, +/-2) points).  Run where the reference sources are present:
    make -C oracle ref && python tests/golden/make_decode_golden.py
"""
import json
import os
import random
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from oracle import Oracle, Reference, build  # noqa: E402

P = 0x1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "decode.json")


def be(x):
    return x.to_bytes(48, "big")


def sqrt_p(a):
    s = pow(a, (P + 1) // 4, P)
    return s if s * s % P == a % P else None


def encodings(o):
    rnd = random.Random(2026)
    enc48, enc96 = [], []
    pts = o.gen_points(77, 40)
    for i in range(40):
        a = pts[96 * i:96 * i + 96]
        jac = o.from_affine(a)
        enc48.append(o.compress(jac))
        enc96.append(o.serialize(jac))
    # infinity encodings, good and bad
    enc48 += [bytes([0xC0]) + bytes(47), bytes([0xE0]) + bytes(47), bytes([0xC0]) + bytes(46) + b"\x01",
              bytes([0x40]) + bytes(47), bytes(48), bytes([0x80]) + bytes(47), bytes([0xC1]) + bytes(47)]
    enc96 += [bytes([0x40]) + bytes(95), bytes([0x60]) + bytes(95), bytes([0x40]) + bytes(94) + b"\x01",
              bytes(96), bytes([0x20]) + bytes(95), bytes([0xC0]) + bytes(95)]
    # non-canonical x / y
    for x in (P, P + 1, (1 << 381) - 1):
        enc48.append(bytes([be(x)[0] | 0x80]) + be(x)[1:])
        enc96.append(be(x) + be(2))
        enc96.append(be(1) + be(x))
    # top-bit conveying: flags cleared from x before the range check
    # off-curve x (x^3 + 4 not a square) and on-curve non-subgroup points
    off, on = [], []
    while len(off) < 20 or len(on) < 30:
        x = rnd.randrange(P)
        y = sqrt_p((x * x * x + 4) % P)
        if y is None and len(off) < 20:
            off.append(x)
        elif y is not None and len(on) < 30:
            on.append((x, y))
    for x in off:
        e = bytearray(be(x))
        e[0] |= 0x80 | (0x20 if rnd.random() < 0.5 else 0)
        enc48.append(bytes(e))
        enc96.append(be(x) + be(rnd.randrange(P)))
    for x, y in on:
        for yy in (y, P - y):
            e = bytearray(be(x))
            e[0] |= 0x80 | (0x20 if yy > (P - 1) // 2 else 0)
            enc48.append(bytes(e))
            enc96.append(be(x) + be(yy))
    # valid x with a wrong y (off-curve uncompressed)
    for i in range(5):
        s = bytearray(enc96[i])
        s[95] ^= 1
        enc96.append(bytes(s))
    # the (0, +/-2) points
    enc48 += [bytes([0x80]) + bytes(47), bytes([0xA0]) + bytes(47)]
    enc96 += [be(0) + be(2), be(0) + be(P - 2)]
    return enc48, enc96


def main():
    build(ref=True)
    o, r = Oracle(), Reference()
    enc48, enc96 = encodings(o)
    init = bytes(range(96))
    g = {"uncompress": [], "deserialize": [], "in_g1": []}
    for e in enc48:
        err, out = r.uncompress(e, init)
        g["uncompress"].append({"in": e.hex(), "err": err, "out": out.hex()})
    for e in enc96:
        err, out = r.deserialize(e, init)
        g["deserialize"].append({"in": e.hex(), "err": err, "out": out.hex()})
    # membership of every successfully decoded point (and of infinity)
    seen = set()
    for c in g["uncompress"] + g["deserialize"]:
        if c["err"] == 0 and c["out"] not in seen:
            seen.add(c["out"])
            g["in_g1"].append({"point": c["out"], "in_g1": r.in_g1(bytes.fromhex(c["out"]))})
    json.dump(g, open(OUT, "w"), indent=1)
    print({k: len(v) for k, v in g.items()}, "errors:",
          sorted({c["err"] for c in g["uncompress"] + g["deserialize"]}),
          "non-member:", sum(1 for c in g["in_g1"] if not c["in_g1"]))


if __name__ == "__main__":
    main()
