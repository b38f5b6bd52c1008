"""The G1 FFT stage kernel's thread-to-butterfly mapping (fft.cu
k_fft_stage_multi), restated in Python: for every job shape and stage level,
the threads of a launch cover each butterfly of the level's active groups
exactly once with in-bounds element indices, trivial (j = 0) butterflies come
after the non-trivial ones, and where a job takes the one-root-per-warp form
(one lane per butterfly, a multiple of 32 active groups) every aligned warp of
its non-trivial range holds a single root.  No GPU involved."""


def brev(x, bits):
    return int(format(x, "0%db" % bits)[::-1], 2) if bits else 0


def level_map(n, xn, length, quad):
    """(g, j, shared) per thread index b of one job at one level."""
    logn, loglen = n.bit_length() - 1, length.bit_length() - 1
    half, groups = length // 2, n // length
    active = min(groups, xn)
    nontriv = active * (half - 1)
    out = []
    for b in range(active * half):
        shared = False
        if b < nontriv:
            if not quad and active % 32 == 0:
                j, g, shared = 1 + b // active, b % active, True
            else:
                g, j = b // (half - 1), 1 + b % (half - 1)
        else:
            g, j = b - nontriv, 0
        if active < groups:
            g = brev(g, logn - loglen)
        out.append((g, j, shared))
    return out


def active_groups(n, xn, length):
    """Groups holding a non-identity input after the bit-reversal permutation."""
    logn, loglen = n.bit_length() - 1, length.bit_length() - 1
    groups = n // length
    return {g for g in range(groups) if brev(g, logn - loglen) < xn} if xn < groups else set(range(groups))


def test_stage_mapping_covers_each_butterfly_once():
    shapes = [(n, xn) for n in (32, 1024, 4096, 1 << 14) for xn in (1, 5, 31, 32, 33, 64, 100, 512, 513, 8192, n)
              if xn <= n]
    for n, xn in shapes:
        length = 2
        while length <= n:
            for quad in (False, True):
                m = level_map(n, xn, length, quad)
                seen = set()
                for g, j, _ in m:
                    i0 = g * length + j
                    assert 0 <= j < length // 2 and i0 + length // 2 < n
                    seen.add((g, j))
                assert len(seen) == len(m), (n, xn, length)
                assert seen == {(g, j) for g in active_groups(n, xn, length) for j in range(length // 2)}
                js = [j for _, j, _ in m]
                first_trivial = js.index(0) if 0 in js else len(js)
                assert all(j == 0 for j in js[first_trivial:]), (n, xn, length)
            length *= 2


def test_shared_warps_hold_one_root():
    for n, xn in ((1024, 1024), (1 << 16, 1 << 16), (1 << 16, 8192), (4096, 64)):
        length = 2
        while length <= n:
            m = level_map(n, xn, length, False)
            for w in range(0, len(m), 32):
                lanes = m[w:w + 32]
                if all(s for _, _, s in lanes):
                    assert len({j for _, j, _ in lanes}) == 1, (n, xn, length, w)
            length *= 2
    # the 2^16 transform with 8192 inputs takes the shared form over bit-reversed groups at level 2
    m = level_map(1 << 16, 8192, 4, False)
    assert all(s for _, _, s in m[:8192]) and 8192 < (1 << 16) // 4
