"""Regenerate tests/golden/golden.json from the REFERENCE library.

Run in a tree where the reference sources are present:
    make -C oracle ref && python tests/golden/make_golden.py [--large]

Inputs are seeded (oracle.gen_* / synth.py); outputs come from the
reference's own C ABI built from its sources (oracle/_ref/libblst_ref.so):
  * msm:  blst_p1s_mult_pippenger -> blst_p1_compress (48 bytes, hex)
  * fft:  blst_p1_fft / blst_p1_fft_with_domain / blst_p1_ifft_unscaled_with_domain
          -> blst_p1_serialize of every element; small n stored in full,
          larger n as sha256 of the concatenation
  * domain: blst_fr_fft_domain_init bytes (sha256) per size
  * msm_fr: blst_p1s_mult_pippenger_fr (Montgomery Fr scalars) -> compressed
  * fr_fft: blst_fr_fft / blst_fr_fft_with_domain output bytes (sha256)
  * wbits:  blst_p1s_mult_wbits_precompute table bytes (sha256) and
            blst_p1s_mult_wbits -> compressed, per (n, wbits, nbits)

  * msm_fr_variants: blst_p1s_mult_fr and blst_p1s_mult_batch_affine_fr ->
            compressed, and the reference's scratch-size queries for both

  * tile:   blst_p1s_tile_pippenger -> compressed, per (n, nbits, bit0, window)

  * fft_truncated: the reference's fft_forward_truncated_prefix template (C
            entry in oracle/ref_shim.cpp) -> sha256 of blst_p1_serialize of
            every element, per (seed, n, xn); each equals the full transform

  * msm_large: the large-MSM workload's other scalar distributions at 2^20
            and 2^22 (64-bit scalars at nbits = 255 and packed at nbits = 64;
            10% zero scalars with 5% duplicated points), appended to msm
  * fft_large: G1 FFT at 2^14 and 2^16 in all five modes, appended to fft
  * batch_commitments: the batched-commitments workload (1024 commitments,
            k_j = floor(2^U), U ~ U[8, 12] from numpy's default_rng(3), over
            the 4096-point basis P_i = k_i G with k = synth.point_scalars(3),
            scalars synth.scalars(3003)): blst_p1s_mult_pippenger over the
            first k_j basis points -> compressed, every commitment
  * bench_fft: the batched-FFT workload's inputs (the first n points of
            synth.point_scalars(4, 2^16) as Jacobian with z = 1, prepared
            domains) -> sha256 of the forward and inverse outputs per size

`--section wbits|msm_fr_variants|tile|fft_truncated|msm_large|fft_large|batch_commitments|bench_fft`
regenerates only that section of an existing file (msm_large and fft_large
replace their own cases inside msm and fft).  The large sections run their
reference calls on a thread pool (ctypes releases the GIL; the reference has
no global mutable state).
"""
import concurrent.futures as cf
import hashlib
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from oracle import Oracle, Reference, build  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")


def msm_inputs(o, seed, n, kind, nbits, dup):
    pts = o.gen_points(seed, n)
    if dup:
        pts = o.duplicate_points(seed, n, pts)
    sc = o.gen_scalars(seed + 1000, n, kind)
    nbytes = (nbits + 7) // 8
    packed = b"".join(sc[32 * i:32 * i + nbytes] for i in range(n)) if nbytes != 32 else sc
    return pts, packed


def wbits_inputs(o, seed, n, kind, nbits, dup, inf):
    """Seeded points (optionally with duplicates and one point at infinity,
    index seed % n) and packed ceil(nbits/8)-byte scalars."""
    pts, sc = msm_inputs(o, seed, n, kind, nbits, dup)
    if inf:
        k = seed % n
        pts = pts[:96 * k] + bytes(96) + pts[96 * (k + 1):]
    return pts, sc


WBITS_CASES = [
    # (seed, n, wbits, kind, nbits, dup, inf)
    (61, 1, 2, 0, 255, False, False), (62, 5, 2, 0, 255, False, False),
    (63, 17, 3, 0, 255, False, True), (64, 100, 4, 1, 64, False, True),
    (65, 256, 8, 2, 255, True, False), (66, 33, 14, 0, 255, False, False),
    (67, 1000, 6, 0, 256, False, True), (68, 4096, 5, 0, 255, False, False),
    (69, 9, 10, 0, 7, False, False), (70, 8193, 3, 0, 255, False, True),
    (71, 300, 7, 0, 17, True, True), (72, 2, 13, 0, 128, False, False),
]


def wbits_section(o, r):
    out = []
    for seed, n, w, kind, nbits, dup, inf in WBITS_CASES:
        t = time.time()
        pts, sc = wbits_inputs(o, seed, n, kind, nbits, dup, inf)
        table = r.wbits_table(pts, n, w)
        assert len(table) == 96 * n << (w - 1)
        res = r.wbits_msm(table, w, n, sc, nbits)
        out.append({"seed": seed, "n": n, "wbits": w, "kind": kind, "nbits": nbits, "dup": dup, "inf": inf,
                    "table_sha256": hashlib.sha256(table).hexdigest(), "compressed": res.hex()})
        print("wbits", seed, n, w, nbits, res.hex()[:16], "%.1fs" % (time.time() - t), flush=True)
    return out


FR_VARIANT_CASES = [
    # (api, seed, n, window, batch, inf)
    ("mult_fr", 81, 1, 0, 0, False), ("mult_fr", 82, 2, 0, 0, False), ("mult_fr", 83, 100, 0, 0, True),
    ("mult_fr", 84, 4096, 0, 0, False), ("mult_fr", 85, 5000, 0, 0, False), ("mult_fr", 86, 4096, 0, 0, True),
    ("mult_fr", 87, 1 << 15, 0, 0, False),
    ("batch_affine_fr", 91, 1, 5, 128, False), ("batch_affine_fr", 92, 2, 1, 128, False),
    ("batch_affine_fr", 93, 100, 5, 384, False), ("batch_affine_fr", 94, 1000, 10, 128, False),
    ("batch_affine_fr", 95, 4096, 13, 384, False),
]


def fr_variants_section(o, r):
    out = {"cases": [], "mult_fr_scratch": [], "batch_affine_scratch": []}
    for api, seed, n, w, b, inf in FR_VARIANT_CASES:
        pts = o.gen_points(seed, n)
        if inf:
            k = seed % n
            pts = pts[:96 * k] + bytes(96) + pts[96 * (k + 1):]
        frs = b"".join(o.fr_to_mont(o.gen_scalars(seed + 1000, n, 0)[32 * i:32 * i + 32]) for i in range(n))
        res = r.mult_fr(pts, frs, n) if api == "mult_fr" else r.batch_affine_fr(pts, frs, n, w, b)
        out["cases"].append({"api": api, "seed": seed, "n": n, "window": w, "batch": b, "inf": inf,
                             "compressed": res.hex()})
        print(api, seed, n, w, b, res.hex()[:16], flush=True)
    for n in (0, 1, 2, 100, 4095, 4096, 4097, 1 << 14, (1 << 14) + 1, 1 << 15, 1 << 16, 1 << 17, 1 << 18,
              (1 << 18) + 1, 1 << 20, 1 << 22):
        out["mult_fr_scratch"].append([n, r.L.blst_p1s_mult_fr_scratch_sizeof(n)])
    for n in (0, 1, 2, 3, 1000, (1 << 32) - 1, 1 << 32):
        for w in (0, 1, 2, 10, 24, 25):
            for b in (0, 100, 128, 384, 512):
                out["batch_affine_scratch"].append([n, w, b, r.L.blst_p1s_mult_batch_affine_fr_scratch_sizeof(n, w, b)])
    return out


TILE_CASES = [
    # (seed, n, kind, nbits, dup, bit0, window)
    (101, 1, 0, 255, False, 0, 4), (102, 100, 0, 255, False, 0, 8), (103, 100, 0, 255, False, 250, 8),
    (104, 100, 0, 255, False, 254, 8), (105, 1000, 0, 255, False, 100, 13), (106, 1000, 1, 64, False, 60, 10),
    (107, 257, 0, 7, False, 3, 3), (108, 500, 2, 255, False, 17, 1), (109, 4096, 0, 255, False, 128, 16),
    (110, 300, 0, 256, False, 255, 5), (111, 2000, 2, 255, True, 40, 18), (112, 50, 0, 17, False, 0, 17),
]


def tile_section(o, r):
    out = []
    for seed, n, kind, nbits, dup, bit0, window in TILE_CASES:
        pts, sc = msm_inputs(o, seed, n, kind, nbits, dup)
        res = r.tile(pts, sc, n, nbits, bit0, window)
        out.append({"seed": seed, "n": n, "kind": kind, "nbits": nbits, "dup": dup, "bit0": bit0,
                    "window": window, "compressed": res.hex()})
        print("tile", seed, n, nbits, bit0, window, res.hex()[:16], flush=True)
    return out


def fft_truncated_section(o, r):
    """Truncated-prefix forward G1 FFT (the reference's C++ template through
    oracle/ref_shim.cpp): seeded Jacobian inputs with [xn, n) the identity,
    the domain's roots.  Each case also checks the reference's own property
    that the output equals its full forward transform."""
    out = []
    # 2^16 with xn = 8192: half the groups of the second level active (the GPU
    # puts the lanes of a warp on one root over bit-reversed groups there)
    for seed, n, xns in ((41, 32, (1, 5, 13, 24, 32)), (42, 1024, (1, 2, 3, 100, 511, 512, 513, 1000, 1024)),
                         (43, 4096, (1, 7, 1024, 2049, 4096)), (44, 1 << 16, (8192,))):
        d = r.domain(n)
        base = o.jacobian_randomize(seed, n, o.gen_points(seed, n))
        for xn in xns:
            t = time.time()
            jac = base[:144 * xn] + bytes(144 * (n - xn))
            ok, tr = r.p1_fft_truncated_prefix(jac, n, xn, d, n + 2)
            ok2, full = r.p1_fft_with_domain(jac, n, d, n + 2, False)
            assert ok and ok2
            ser = b"".join(r.serialize(tr[144 * i:144 * i + 144]) for i in range(n))
            assert ser == b"".join(r.serialize(full[144 * i:144 * i + 144]) for i in range(n))
            out.append({"seed": seed, "n": n, "xn": xn, "sha256": hashlib.sha256(ser).hexdigest()})
            print("fft_truncated", seed, n, xn, "%.1fs" % (time.time() - t), flush=True)
    return out


MSM_LARGE_CASES = [
    # (seed, n, kind, nbits, dup): the large-MSM workload's distributions (b) and (c)
    (25, 1 << 20, 1, 255, False), (26, 1 << 20, 1, 64, False), (27, 1 << 20, 2, 255, True),
    (28, 1 << 22, 1, 255, False), (29, 1 << 22, 1, 64, False), (30, 1 << 22, 2, 255, True),
]
FFT_LARGE_CASES = [(46, 1 << 14), (47, 1 << 16)]
FFT_MODES = ("fwd", "inv", "dfwd", "dinv", "dunscaled")
_THREADS = max(1, os.cpu_count() or 1)


def _fft_mode(r, jac, n, d, mode):
    if mode == "fwd":
        return r.p1_fft(jac, n, False)
    if mode == "inv":
        return r.p1_fft(jac, n, True)
    if mode == "dfwd":
        return r.p1_fft_with_domain(jac, n, d, n + 2, False)
    if mode == "dinv":
        return r.p1_fft_with_domain(jac, n, d, n + 2, True)
    return r.p1_ifft_unscaled_with_domain(jac, n, d, n + 2)


def msm_large_section(o, r):
    """Reference MSMs of MSM_LARGE_CASES, several at once."""
    def one(case):
        seed, n, kind, nbits, dup = case
        t = time.time()
        pts, sc = msm_inputs(o, seed, n, kind, nbits, dup)
        res = r.msm(pts, sc, n, nbits)
        print("msm_large", seed, n, kind, nbits, dup, res.hex()[:16], "%.1fs" % (time.time() - t), flush=True)
        return {"seed": seed, "n": n, "kind": kind, "nbits": nbits, "dup": dup, "compressed": res.hex()}
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        return list(ex.map(one, MSM_LARGE_CASES))


def fft_large_section(o, r):
    """Reference G1 FFTs of FFT_LARGE_CASES in all five modes, in parallel."""
    inputs = {}
    for seed, n in FFT_LARGE_CASES:
        inputs[(seed, n)] = (o.jacobian_randomize(seed, n, o.gen_points(seed, n)), r.domain(n))

    def one(job):
        (seed, n), mode = job
        t = time.time()
        jac, d = inputs[(seed, n)]
        ok, out = _fft_mode(r, jac, n, d, mode)
        assert ok
        ser = b"".join(r.serialize(out[144 * i:144 * i + 144]) for i in range(n))
        print("fft_large", seed, n, mode, "%.1fs" % (time.time() - t), flush=True)
        return {"seed": seed, "n": n, "mode": mode, "sha256": hashlib.sha256(ser).hexdigest()}
    jobs = [(c, m) for c in FFT_LARGE_CASES for m in FFT_MODES]
    with cf.ThreadPoolExecutor(max_workers=_THREADS) as ex:
        return list(ex.map(one, jobs))


def batch_commitments_inputs(o):
    """The batched-commitments workload: (counts, basis points, scalars)."""
    import numpy as np
    synth = _synth()
    nb, nmsm, seed = 4096, 1024, 3
    rng = np.random.default_rng(seed)
    counts = [int(2 ** u) for u in rng.uniform(8, 12, nmsm)]
    pts = o.points_from_scalars(synth.point_scalars(seed, nb), nb)
    sc = synth.scalars(seed + 3000, sum(counts), 0)
    return counts, pts, sc


def batch_commitments_section(o, r):
    counts, pts, sc = batch_commitments_inputs(o)
    offs = [0]
    for k in counts:
        offs.append(offs[-1] + k)

    def one(j):
        k = counts[j]
        return r.msm(pts[:96 * k], sc[32 * offs[j]:32 * offs[j + 1]], k, 256).hex()
    t = time.time()
    with cf.ThreadPoolExecutor(max_workers=_THREADS) as ex:
        res = list(ex.map(one, range(len(counts))))
    print("batch_commitments", len(res), "%.1fs" % (time.time() - t), flush=True)
    return {"n_basis": 4096, "seed": 3, "nbits": 256, "counts": counts, "compressed": res,
            "sha256": hashlib.sha256(b"".join(bytes.fromhex(x) for x in res)).hexdigest()}


def bench_fft_section(o, r):
    synth = _synth()
    big = 1 << 16
    aff = o.points_from_scalars(synth.point_scalars(4, big), big)
    one_m = ((1 << 384) % 0x1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab
             ).to_bytes(48, "little")

    def one(job):
        n, inverse = job
        t = time.time()
        jac = b"".join(aff[96 * i:96 * i + 96] + one_m for i in range(n))
        ok, out = r.p1_fft_with_domain(jac, n, r.domain(n), n + 2, inverse)
        assert ok
        ser = b"".join(r.serialize(out[144 * i:144 * i + 144]) for i in range(n))
        print("bench_fft", n, inverse, "%.1fs" % (time.time() - t), flush=True)
        return {"n": n, "mode": "dinv" if inverse else "dfwd", "sha256": hashlib.sha256(ser).hexdigest()}
    jobs = [(1 << e, inv) for e in (10, 12, 14, 16) for inv in (False, True)]
    with cf.ThreadPoolExecutor(max_workers=_THREADS) as ex:
        return {"seed": 4, "z": 1, "cases": list(ex.map(one, jobs))}


def _synth():
    import importlib.util
    path = os.path.join(ROOT, "temp-cat-blst_gb300", "synth.py")
    spec = importlib.util.spec_from_file_location("catmsm_synth", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _replace_cases(old, new, key):
    have = {key(c) for c in new}
    return [c for c in old if key(c) not in have] + new


def main():
    large = "--large" in sys.argv
    build(ref=True)
    o, r = Oracle(), Reference()
    if "--section" in sys.argv:
        name = sys.argv[sys.argv.index("--section") + 1]
        g = json.load(open(OUT))
        if name == "msm_large":
            g["msm"] = _replace_cases(g["msm"], msm_large_section(o, r), lambda c: (c["seed"], c["n"]))
        elif name == "fft_large":
            g["fft"] = _replace_cases(g["fft"], fft_large_section(o, r), lambda c: (c["seed"], c["n"], c["mode"]))
        else:
            g[name] = {"wbits": wbits_section, "msm_fr_variants": fr_variants_section, "tile": tile_section,
                       "fft_truncated": fft_truncated_section, "batch_commitments": batch_commitments_section,
                       "bench_fft": bench_fft_section}[name](o, r)
        json.dump(g, open(OUT, "w"), indent=1)
        print("wrote", OUT)
        return
    g = {"msm": [], "fft": [], "domain": []}
    cases = [
        # (seed, n, kind, nbits, dup)
        (11, 1, 0, 255, False), (12, 2, 0, 255, False), (13, 3, 0, 255, False),
        (14, 17, 0, 255, False), (15, 100, 0, 255, False), (16, 100, 0, 256, False),
        (17, 100, 0, 64, False), (18, 100, 0, 1, False), (19, 100, 0, 7, False),
        (20, 100, 0, 17, False), (21, 100, 0, 128, False), (22, 257, 1, 64, False),
        (23, 1000, 2, 255, True), (24, 999, 0, 200, False),
        (1, 4096, 0, 255, False),                      # plain MSM, n = 4096, seed 1
        (2, 1 << 16, 0, 255, False), (3, 1 << 16, 1, 64, False), (4, 1 << 16, 2, 255, True),
        (5, 1 << 16, 1, 255, False),
    ]
    if large:
        cases += [(6, 1 << 20, 0, 255, False), (7, 1 << 22, 0, 255, False)]
    for seed, n, kind, nbits, dup in cases:
        t = time.time()
        pts, sc = msm_inputs(o, seed, n, kind, nbits, dup)
        res = r.msm(pts, sc, n, nbits)
        g["msm"].append({"seed": seed, "n": n, "kind": kind, "nbits": nbits, "dup": dup,
                         "compressed": res.hex()})
        print("msm", seed, n, kind, nbits, dup, res.hex()[:16], "%.1fs" % (time.time() - t), flush=True)

    for k in range(0, 17):
        n = 1 << k
        g["domain"].append({"n": n, "sha256": hashlib.sha256(r.domain(n)).hexdigest()})

    fft_cases = [(31, 1), (32, 2), (33, 4), (34, 8), (35, 16), (36, 64), (37, 256), (38, 1024)]
    if large:
        fft_cases += [(39, 4096)]
    for seed, n in fft_cases:
        aff = o.gen_points(seed, n)
        jac = o.jacobian_randomize(seed, n, aff)
        d = r.domain(n)
        for mode in ("fwd", "inv", "dfwd", "dinv", "dunscaled"):
            t = time.time()
            if mode == "fwd":
                ok, out = r.p1_fft(jac, n, False)
            elif mode == "inv":
                ok, out = r.p1_fft(jac, n, True)
            elif mode == "dfwd":
                ok, out = r.p1_fft_with_domain(jac, n, d, n + 2, False)
            elif mode == "dinv":
                ok, out = r.p1_fft_with_domain(jac, n, d, n + 2, True)
            else:
                ok, out = r.p1_ifft_unscaled_with_domain(jac, n, d, n + 2)
            assert ok
            ser = b"".join(r.serialize(out[144 * i:144 * i + 144]) for i in range(n))
            entry = {"seed": seed, "n": n, "mode": mode, "sha256": hashlib.sha256(ser).hexdigest()}
            if n <= 16:
                entry["serialized"] = ser.hex()
            g["fft"].append(entry)
            print("fft", seed, n, mode, "%.1fs" % (time.time() - t), flush=True)
    # Fr-scalar MSM (blst_p1s_mult_pippenger_fr): Montgomery Fr scalars
    g["msm_fr"] = []
    for seed, n in ((41, 1), (42, 2), (43, 100), (44, 4096), (45, 1 << 14)):
        pts = o.gen_points(seed, n)
        frs = b"".join(o.fr_to_mont(o.gen_scalars(seed + 1000, n, 0)[32 * i:32 * i + 32]) for i in range(n))
        g["msm_fr"].append({"seed": seed, "n": n, "compressed": r.msm_fr(pts, frs, n).hex()})
        print("msm_fr", seed, n, flush=True)
    # Fr FFT (blst_fr_fft / blst_fr_fft_with_domain): values = seeded Fr in Montgomery form
    g["fr_fft"] = []
    for seed, n in ((51, 1), (52, 2), (53, 8), (54, 256), (55, 2048), (56, 4096), (57, 1 << 16)):
        vals = b"".join(o.fr_to_mont(o.gen_scalars(seed, n, 0)[32 * i:32 * i + 32]) for i in range(n))
        d = r.domain(n)
        for mode in ("fwd", "inv", "dfwd", "dinv"):
            if mode == "fwd":
                ok, out = r.fr_fft(vals, n, False)
            elif mode == "inv":
                ok, out = r.fr_fft(vals, n, True)
            elif mode == "dfwd":
                ok, out = r.fr_fft_with_domain(vals, n, d, n + 2, False)
            else:
                ok, out = r.fr_fft_with_domain(vals, n, d, n + 2, True)
            assert ok
            g["fr_fft"].append({"seed": seed, "n": n, "mode": mode, "sha256": hashlib.sha256(out).hexdigest()})
        print("fr_fft", seed, n, flush=True)
    g["wbits"] = wbits_section(o, r)
    g["msm_fr_variants"] = fr_variants_section(o, r)
    g["tile"] = tile_section(o, r)
    g["fft_truncated"] = fft_truncated_section(o, r)
    if large:
        g["msm"] += msm_large_section(o, r)
        g["fft"] += fft_large_section(o, r)
        g["batch_commitments"] = batch_commitments_section(o, r)
        g["bench_fft"] = bench_fft_section(o, r)
    elif os.path.exists(OUT):
        # keep previously generated large cases and sections
        old = json.load(open(OUT))
        have = {(c["seed"], c["n"]) for c in g["msm"]}
        g["msm"] += [c for c in old["msm"] if (c["seed"], c["n"]) not in have]
        havef = {(c["seed"], c["n"], c["mode"]) for c in g["fft"]}
        g["fft"] += [c for c in old["fft"] if (c["seed"], c["n"], c["mode"]) not in havef]
        for name in ("batch_commitments", "bench_fft"):
            if name in old:
                g[name] = old[name]
    json.dump(g, open(OUT, "w"), indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
