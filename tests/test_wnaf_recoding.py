"""The width-5 NAF recoding of a GLV half (curve.cuh wnaf5_128), restated
word for word in Python: five 32-bit words, the low five bits as the digit,
the carry of a negative digit through the words, a one-bit shift per digit.
Checks the properties the FFT's shared-root scalar multiplication relies on:
the digits rebuild the value, every digit is 0 or odd in [-15, 15], at most
one nonzero digit in any five consecutive positions, and at most 129 digits
(the digit buffer holds 130).  No GPU involved."""
import random

M32 = (1 << 32) - 1


def wnaf5_128(k):
    w = [(k >> (32 * i)) & M32 for i in range(4)] + [0]
    digits = []
    for _ in range(130):
        if not any(w):
            break
        v = 0
        if w[0] & 1:
            v = w[0] & 31
            if v > 16:
                v -= 32
            if v > 0:
                w[0] = (w[0] - v) & M32
            else:
                s = w[0] + (-v)
                w[0] = s & M32
                for i in (1, 2, 3):
                    s = (s >> 32) + w[i]
                    w[i] = s & M32
                w[4] = (w[4] + (s >> 32)) & M32
        digits.append(v)
        for i in range(4):
            w[i] = ((w[i] >> 1) | (w[i + 1] << 31)) & M32
        w[4] >>= 1
    assert not any(w), "value left after 130 digits"
    return digits


def test_wnaf5_properties():
    rnd = random.Random(5)
    top = (1 << 128) - 1
    vals = [0, 1, 2, 3, 15, 16, 17, 31, 32, 33, top, top - 1, top - 15, 1 << 127, (1 << 127) - 1,
            0x5555555555555555_5555555555555555, 0xAAAAAAAAAAAAAAAA_AAAAAAAAAAAAAAAA, (1 << 96) - 1, (1 << 64) - 1]
    vals += [rnd.randrange(1 << 128) for _ in range(20000)]
    vals += [rnd.randrange(1 << rnd.randrange(1, 129)) for _ in range(5000)]
    worst = 0
    for k in vals:
        d = wnaf5_128(k)
        assert sum(x << i for i, x in enumerate(d)) == k, hex(k)
        assert all(x == 0 or (x % 2 == 1 and -15 <= x <= 15) for x in d), hex(k)
        nz = [i for i, x in enumerate(d) if x]
        assert all(b - a >= 5 for a, b in zip(nz, nz[1:])), hex(k)
        assert not d or d[-1] != 0, hex(k)
        worst = max(worst, len(d))
    assert worst <= 129
    # a carry past 2^128 happens: 2^128 - 1 recodes to 2^128 - 1 with 129 digits
    assert len(wnaf5_128(top)) == 129


def test_wnaf5_density():
    """~1/6 of the positions of a random 128-bit half are nonzero, so two
    halves cost ~43 additions against ~50 for the 5-bit fixed windows."""
    rnd = random.Random(6)
    total = sum(sum(1 for x in wnaf5_128(rnd.randrange(1 << 128)) if x) for _ in range(2000))
    assert 20.5 < total / 2000 < 22.5
