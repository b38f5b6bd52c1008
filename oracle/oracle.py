"""ctypes access to the CPU oracle libraries (test infrastructure only).

* ``Oracle``     -- the C restatement in this directory (liboracle.so).
* ``Reference``  -- the reference library compiled from its own sources
                    (oracle/_ref/libblst_ref.so), present only where the
                    reference tree was available at build time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module.  All buffers are plain ``bytes``/``bytearray`` in the reference ABI
layouts: 96-byte affine points, 144-byte Jacobian points, 32-byte scalars,
32-byte Montgomery Fr values.
"""
import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libblst_ref.so")

P1 = 144
P1A = 96
FR = 32

_vp = C.c_void_p
_sz = C.c_size_t


# Where the reference sources are read from when the reference library is
# built (BLST_REFERENCE_DIR; the default is this build machine's checkout).
REFERENCE_DIR = os.environ.get("BLST_REFERENCE_DIR", "/root/reference")


def build(ref=False):
    """Compile liboracle.so (and the reference .so if asked and the reference
    sources are present)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref and os.path.isdir(REFERENCE_DIR):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "-j8", "REF=" + REFERENCE_DIR], check=True)


def _buf(data):
    if isinstance(data, bytearray):
        return (C.c_char * len(data)).from_buffer(data)
    return C.c_char_p(bytes(data))


class _Common:
    """Shared helpers over a library exposing the reference's C ABI shape."""

    def _ptr_array(self, base, n, stride):
        arr = (C.c_void_p * 2)()
        arr[0] = C.cast(base, C.c_void_p)
        arr[1] = None
        return arr

    def msm(self, points: bytes, scalars: bytes, n: int, nbits: int = 255) -> bytes:
        """Contiguous-descriptor MSM; returns the 48-byte compressed result."""
        pts = bytearray(points)
        scs = bytearray(scalars)
        pbuf = _buf(pts)
        sbuf = _buf(scs)
        parr = (C.c_void_p * 2)(C.cast(pbuf, C.c_void_p), None)
        sarr = (C.c_void_p * 2)(C.cast(sbuf, C.c_void_p), None)
        scratch = (C.c_uint64 * max(1, self.scratch_sizeof(n) // 8 + 1))()
        ret = bytearray(P1)
        self._msm(_buf(ret), parr, n, sarr, nbits, scratch)
        return self.compress(bytes(ret))

    def _bind_wbits(self, prefix):
        L = self.L
        f = lambda name: getattr(L, prefix + name)
        f("p1s_mult_wbits_precompute_sizeof").restype = _sz
        f("p1s_mult_wbits_precompute_sizeof").argtypes = [_sz, _sz]
        f("p1s_mult_wbits_precompute").argtypes = [_vp, _sz, _vp, _sz]
        f("p1s_mult_wbits_scratch_sizeof").restype = _sz
        f("p1s_mult_wbits_scratch_sizeof").argtypes = [_sz]
        f("p1s_mult_wbits").argtypes = [_vp, _vp, _sz, _sz, _vp, _sz, _vp]
        self.wbits_table_sizeof = f("p1s_mult_wbits_precompute_sizeof")
        self.wbits_scratch_sizeof = f("p1s_mult_wbits_scratch_sizeof")
        self._wpre = f("p1s_mult_wbits_precompute")
        self._wmsm = f("p1s_mult_wbits")

    def tile(self, points: bytes, scalars: bytes, n: int, nbits: int, bit0: int, window: int) -> bytes:
        """One signed window (p1s_tile_pippenger, contiguous descriptors) -> compressed."""
        f = getattr(self.L, ("oracle_" if isinstance(self, Oracle) else "blst_") + "p1s_tile_pippenger")
        f.argtypes = [_vp, _vp, _sz, _vp, _sz, _vp, _sz, _sz]
        pbuf, sbuf = _buf(bytearray(points)), _buf(bytearray(scalars))
        parr = (C.c_void_p * 2)(C.cast(pbuf, C.c_void_p), None)
        sarr = (C.c_void_p * 2)(C.cast(sbuf, C.c_void_p), None)
        scratch = (C.c_uint64 * ((192 << max(0, window - 1)) // 8 + 1))()
        ret = bytearray(P1)
        f(_buf(ret), parr, n, sarr, nbits, scratch, bit0, window)
        return self.compress(bytes(ret))

    def wbits_table(self, points: bytes, n: int, wbits: int) -> bytes:
        """Contiguous-descriptor table precompute; returns the table bytes."""
        size = self.wbits_table_sizeof(wbits, n)
        table = bytearray(size)
        pbuf = _buf(bytearray(points))
        parr = (C.c_void_p * 2)(C.cast(pbuf, C.c_void_p), None)
        self._wpre(_buf(table), wbits, parr, n)
        return bytes(table)

    def wbits_msm(self, table: bytes, wbits: int, n: int, scalars: bytes, nbits: int = 255) -> bytes:
        """Contiguous-descriptor fixed-table MSM; returns the compressed result."""
        sbuf = _buf(bytearray(scalars))
        sarr = (C.c_void_p * 2)(C.cast(sbuf, C.c_void_p), None)
        scratch = (C.c_uint64 * max(1, self.wbits_scratch_sizeof(n) // 8))()
        ret = bytearray(P1)
        self._wmsm(_buf(ret), _buf(bytearray(table)), wbits, n, sarr, nbits, scratch)
        return self.compress(bytes(ret))


class Oracle(_Common):
    def __init__(self, path=ORACLE_SO):
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        self.L = L
        L.oracle_init()
        L.oracle_p1s_mult_pippenger_scratch_sizeof.restype = _sz
        L.oracle_p1s_mult_pippenger_scratch_sizeof.argtypes = [_sz]
        L.oracle_p1s_mult_pippenger.argtypes = [_vp, _vp, _sz, _vp, _sz, _vp]
        L.oracle_p1s_mult_pippenger_window.argtypes = [_vp, _vp, _sz, _vp, _sz, _vp, _sz]
        L.oracle_p1s_mult_naive.argtypes = [_vp, _vp, _sz, _vp, _sz]
        L.oracle_p1s_tile_pippenger.argtypes = [_vp, _vp, _sz, _vp, _sz, _vp, _sz, _sz]
        L.oracle_pippenger_window_size.restype = _sz
        L.oracle_pippenger_window_size.argtypes = [_sz]
        L.op1_compress.argtypes = [_vp, _vp]
        L.op1_serialize.argtypes = [_vp, _vp]
        L.op1_affine_serialize.argtypes = [_vp, _vp]
        L.op1_generator.argtypes = [_vp]
        L.op1_mult_vartime.argtypes = [_vp, _vp, _vp, _sz]
        L.op1_dadd.argtypes = [_vp, _vp, _vp]
        L.op1_from_affine.argtypes = [_vp, _vp]
        L.op1_to_affine.argtypes = [_vp, _vp]
        L.op1_on_curve.restype = C.c_bool
        L.op1_on_curve.argtypes = [_vp]
        L.oracle_fr_fft_domain_len.restype = _sz
        L.oracle_fr_fft_domain_len.argtypes = [_sz]
        for f in ("oracle_fr_fft_domain_init",):
            getattr(L, f).restype = C.c_bool
            getattr(L, f).argtypes = [_vp, _sz, _sz]
        L.oracle_p1_fft.restype = C.c_bool
        L.oracle_p1_fft.argtypes = [_vp, _sz, C.c_bool]
        L.oracle_p1_fft_with_domain.restype = C.c_bool
        L.oracle_p1_fft_with_domain.argtypes = [_vp, _sz, _vp, _sz, C.c_bool]
        L.oracle_p1_ifft_unscaled_with_domain.restype = C.c_bool
        L.oracle_p1_ifft_unscaled_with_domain.argtypes = [_vp, _sz, _vp, _sz]
        L.oracle_p1_fft_truncated_prefix.restype = C.c_bool
        L.oracle_p1_fft_truncated_prefix.argtypes = [_vp, _sz, _sz, _vp, _sz]
        L.oracle_fr_fft.restype = C.c_bool
        L.oracle_fr_fft.argtypes = [_vp, _sz, C.c_bool]
        L.oracle_fr_fft_with_domain.restype = C.c_bool
        L.oracle_fr_fft_with_domain.argtypes = [_vp, _sz, _vp, _sz, C.c_bool]
        L.oracle_gen_scalars.argtypes = [C.c_uint64, _sz, C.c_int, _vp]
        L.oracle_points_from_scalars.argtypes = [_vp, _sz, _vp, C.c_int]
        L.oracle_duplicate_points.argtypes = [C.c_uint64, _sz, _vp]
        L.oracle_jacobian_randomize.argtypes = [C.c_uint64, _sz, _vp, _vp]
        L.ofr_to_mont.argtypes = [_vp, _vp]
        L.ofr_from_mont.argtypes = [_vp, _vp]
        self._msm = L.oracle_p1s_mult_pippenger
        self.scratch_sizeof = L.oracle_p1s_mult_pippenger_scratch_sizeof
        self._bind_wbits("oracle_")
        self.window_size = L.oracle_pippenger_window_size

    # ---- inputs ----
    def gen_scalars(self, seed, n, kind=0) -> bytes:
        out = bytearray(32 * n)
        self.L.oracle_gen_scalars(seed, n, kind, _buf(out))
        return bytes(out)

    def points_from_scalars(self, k32: bytes, n: int, nthreads: int = None) -> bytes:
        out = bytearray(P1A * n)
        nt = nthreads or max(1, min(16, os.cpu_count() or 1))
        self.L.oracle_points_from_scalars(_buf(k32), n, _buf(out), nt)
        return bytes(out)

    def gen_points(self, seed, n, nthreads=None) -> bytes:
        return self.points_from_scalars(self.gen_scalars(seed ^ 0xA5A5A5A5, n, 0), n, nthreads)

    def duplicate_points(self, seed, n, points: bytes) -> bytes:
        b = bytearray(points)
        self.L.oracle_duplicate_points(seed, n, _buf(b))
        return bytes(b)

    def jacobian_randomize(self, seed, n, affine: bytes) -> bytes:
        out = bytearray(P1 * n)
        self.L.oracle_jacobian_randomize(seed, n, _buf(affine), _buf(out))
        return bytes(out)

    # ---- group ----
    def compress(self, p: bytes) -> bytes:
        out = bytearray(48)
        self.L.op1_compress(_buf(out), _buf(p))
        return bytes(out)

    def serialize(self, p: bytes) -> bytes:
        out = bytearray(96)
        self.L.op1_serialize(_buf(out), _buf(p))
        return bytes(out)

    def affine_serialize(self, a: bytes) -> bytes:
        out = bytearray(96)
        self.L.op1_affine_serialize(_buf(out), _buf(a))
        return bytes(out)

    def generator(self) -> bytes:
        out = bytearray(P1)
        self.L.op1_generator(_buf(out))
        return bytes(out)

    def mult(self, p: bytes, scalar: bytes, nbits=256) -> bytes:
        out = bytearray(P1)
        self.L.op1_mult_vartime(_buf(out), _buf(p), _buf(scalar), nbits)
        return bytes(out)

    def add(self, a: bytes, b: bytes) -> bytes:
        out = bytearray(P1)
        self.L.op1_dadd(_buf(out), _buf(a), _buf(b))
        return bytes(out)

    def from_affine(self, a: bytes) -> bytes:
        out = bytearray(P1)
        self.L.op1_from_affine(_buf(out), _buf(a))
        return bytes(out)

    def on_curve(self, p: bytes) -> bool:
        return bool(self.L.op1_on_curve(_buf(p)))

    def msm_seconds(self, points: bytes, scalars: bytes, n: int, nbits: int = 255):
        """One whole contiguous-descriptor MSM call, timed around the C call
        only (buffers prepared outside the timer); returns (seconds,
        compressed result)."""
        import time
        pbuf, sbuf = _buf(bytearray(points)), _buf(bytearray(scalars))
        parr = (C.c_void_p * 2)(C.cast(pbuf, C.c_void_p), None)
        sarr = (C.c_void_p * 2)(C.cast(sbuf, C.c_void_p), None)
        scratch = (C.c_uint64 * max(1, self.scratch_sizeof(n) // 8 + 1))()
        ret = bytearray(P1)
        rb = _buf(ret)
        t = time.perf_counter()
        self._msm(rb, parr, n, sarr, nbits, scratch)
        el = time.perf_counter() - t
        return el, self.compress(bytes(ret))

    def msm_raw(self, ret: bytearray, parr, n, sarr, nbits, scratch):
        self._msm(_buf(ret), parr, n, sarr, nbits, scratch)

    def msm_window(self, points, scalars, n, nbits, window) -> bytes:
        pbuf, sbuf = _buf(bytearray(points)), _buf(bytearray(scalars))
        parr = (C.c_void_p * 2)(C.cast(pbuf, C.c_void_p), None)
        sarr = (C.c_void_p * 2)(C.cast(sbuf, C.c_void_p), None)
        scratch = (C.c_uint64 * ((192 << max(0, window - 1)) // 8 + 1))()
        ret = bytearray(P1)
        self.L.oracle_p1s_mult_pippenger_window(_buf(ret), parr, n, sarr, nbits, scratch, window)
        return self.compress(bytes(ret))

    def tile_seconds(self, points, scalars, n, nbits, bit0, window, reps=1) -> float:
        """Wall time of `reps` single-window tiles (bounded CPU sample)."""
        import time
        pbuf, sbuf = _buf(bytearray(points)), _buf(bytearray(scalars))
        parr = (C.c_void_p * 2)(C.cast(pbuf, C.c_void_p), None)
        sarr = (C.c_void_p * 2)(C.cast(sbuf, C.c_void_p), None)
        scratch = (C.c_uint64 * ((192 << max(0, window - 1)) // 8 + 1))()
        ret = bytearray(P1)
        t = time.perf_counter()
        for _ in range(reps):
            self.L.oracle_p1s_tile_pippenger(_buf(ret), parr, n, sarr, nbits, scratch, bit0, window)
        return time.perf_counter() - t

    def msm_naive(self, points, scalars, n, nbits) -> bytes:
        ret = bytearray(P1)
        self.L.oracle_p1s_mult_naive(_buf(ret), _buf(points), n, _buf(scalars), nbits)
        return self.compress(bytes(ret))

    # ---- FFT ----
    def domain(self, n) -> bytes:
        L = self.L.oracle_fr_fft_domain_len(n)
        out = bytearray(FR * L)
        ok = self.L.oracle_fr_fft_domain_init(_buf(out), L, n)
        assert ok
        return bytes(out)

    def p1_fft(self, values: bytes, n, inverse) -> (bool, bytes):
        b = bytearray(values)
        ok = self.L.oracle_p1_fft(_buf(b), n, inverse)
        return ok, bytes(b)

    def p1_fft_with_domain(self, values, n, domain, domain_len, inverse):
        b = bytearray(values)
        ok = self.L.oracle_p1_fft_with_domain(_buf(b), n, _buf(domain), domain_len, inverse)
        return ok, bytes(b)

    def p1_ifft_unscaled_with_domain(self, values, n, domain, domain_len):
        b = bytearray(values)
        ok = self.L.oracle_p1_ifft_unscaled_with_domain(_buf(b), n, _buf(domain), domain_len)
        return ok, bytes(b)

    def p1_fft_truncated_prefix(self, values, n, xn, domain, domain_len):
        b = bytearray(values)
        ok = self.L.oracle_p1_fft_truncated_prefix(_buf(b), n, xn, _buf(domain), domain_len)
        return ok, bytes(b)

    def fr_fft(self, values: bytes, n, inverse):
        b = bytearray(values)
        ok = self.L.oracle_fr_fft(_buf(b), n, inverse)
        return ok, bytes(b)

    def fr_fft_with_domain(self, values, n, domain, domain_len, inverse):
        b = bytearray(values)
        ok = self.L.oracle_fr_fft_with_domain(_buf(b), n, _buf(domain), domain_len, inverse)
        return ok, bytes(b)

    def msm_fr(self, points: bytes, frs: bytes, n: int) -> bytes:
        """blst_p1s_mult_pippenger_fr semantics: Montgomery Fr scalars."""
        canon = b"".join(self.fr_from_mont(frs[32 * i:32 * i + 32]) for i in range(n))
        return self.msm(points, canon, n, 255)

    def fr_to_mont(self, canon: bytes) -> bytes:
        out = bytearray(32)
        self.L.ofr_to_mont(_buf(out), _buf(canon))
        return bytes(out)

    def fr_from_mont(self, m: bytes) -> bytes:
        out = bytearray(32)
        self.L.ofr_from_mont(_buf(out), _buf(m))
        return bytes(out)


class Reference(_Common):
    """The reference library's own C ABI (compiled from its sources)."""

    def __init__(self, path=REF_SO):
        L = C.CDLL(path)
        self.L = L
        L.blst_p1s_mult_pippenger_scratch_sizeof.restype = _sz
        L.blst_p1s_mult_pippenger_scratch_sizeof.argtypes = [_sz]
        L.blst_p1s_mult_pippenger.argtypes = [_vp, _vp, _sz, _vp, _sz, _vp]
        L.blst_p1s_mult_pippenger_window.argtypes = [_vp, _vp, _sz, _vp, _sz, _vp, _sz]
        L.blst_p1_compress.argtypes = [_vp, _vp]
        L.blst_p1_serialize.argtypes = [_vp, _vp]
        L.blst_p1_affine_serialize.argtypes = [_vp, _vp]
        L.blst_p1_mult.argtypes = [_vp, _vp, _vp, _sz]
        L.blst_p1_add_or_double.argtypes = [_vp, _vp, _vp]
        L.blst_p1_to_affine.argtypes = [_vp, _vp]
        L.blst_p1_from_affine.argtypes = [_vp, _vp]
        L.blst_p1_generator.restype = _vp
        L.blst_fr_fft_domain_len.restype = _sz
        L.blst_fr_fft_domain_len.argtypes = [_sz]
        L.blst_fr_fft_domain_init.restype = C.c_bool
        L.blst_fr_fft_domain_init.argtypes = [_vp, _sz, _sz]
        L.blst_p1_fft.restype = C.c_bool
        L.blst_p1_fft.argtypes = [_vp, _sz, C.c_bool]
        L.blst_p1_fft_with_domain.restype = C.c_bool
        L.blst_p1_fft_with_domain.argtypes = [_vp, _sz, _vp, _sz, C.c_bool]
        L.blst_p1_ifft_unscaled_with_domain.restype = C.c_bool
        L.blst_p1_ifft_unscaled_with_domain.argtypes = [_vp, _sz, _vp, _sz]
        if hasattr(L, "refshim_p1_fft_truncated_prefix"):
            L.refshim_p1_fft_truncated_prefix.restype = C.c_bool
            L.refshim_p1_fft_truncated_prefix.argtypes = [_vp, _sz, _sz, _vp]
        L.blst_fr_fft.restype = C.c_bool
        L.blst_fr_fft.argtypes = [_vp, _sz, C.c_bool]
        L.blst_fr_fft_with_domain.restype = C.c_bool
        L.blst_fr_fft_with_domain.argtypes = [_vp, _sz, _vp, _sz, C.c_bool]
        L.blst_p1_uncompress.restype = C.c_int
        L.blst_p1_uncompress.argtypes = [_vp, _vp]
        L.blst_p1_deserialize.restype = C.c_int
        L.blst_p1_deserialize.argtypes = [_vp, _vp]
        L.blst_p1_affine_in_g1.restype = C.c_bool
        L.blst_p1_affine_in_g1.argtypes = [_vp]
        L.blst_p1s_mult_pippenger_fr_scratch_sizeof.restype = _sz
        L.blst_p1s_mult_pippenger_fr_scratch_sizeof.argtypes = [_sz]
        L.blst_p1s_mult_pippenger_fr.restype = C.c_bool
        L.blst_p1s_mult_pippenger_fr.argtypes = [_vp, _vp, _vp, _sz, _vp, _sz]
        L.blst_p1s_mult_fr_scratch_sizeof.restype = _sz
        L.blst_p1s_mult_fr_scratch_sizeof.argtypes = [_sz]
        L.blst_p1s_mult_fr.restype = C.c_bool
        L.blst_p1s_mult_fr.argtypes = [_vp, _vp, _vp, _sz, _vp, _sz]
        L.blst_p1s_mult_batch_affine_fr_scratch_sizeof.restype = _sz
        L.blst_p1s_mult_batch_affine_fr_scratch_sizeof.argtypes = [_sz, _sz, _sz]
        L.blst_p1s_mult_batch_affine_fr.restype = C.c_bool
        L.blst_p1s_mult_batch_affine_fr.argtypes = [_vp, _vp, _vp, _sz, _vp, _sz, _sz, _sz]
        self._msm = L.blst_p1s_mult_pippenger
        self.scratch_sizeof = L.blst_p1s_mult_pippenger_scratch_sizeof
        self._bind_wbits("blst_")

    def compress(self, p: bytes) -> bytes:
        out = bytearray(48)
        self.L.blst_p1_compress(_buf(out), _buf(p))
        return bytes(out)

    def serialize(self, p: bytes) -> bytes:
        out = bytearray(96)
        self.L.blst_p1_serialize(_buf(out), _buf(p))
        return bytes(out)

    def affine_serialize(self, a: bytes) -> bytes:
        out = bytearray(96)
        self.L.blst_p1_affine_serialize(_buf(out), _buf(a))
        return bytes(out)

    def generator(self) -> bytes:
        return C.string_at(self.L.blst_p1_generator(), P1)

    def mult(self, p: bytes, scalar: bytes, nbits=256) -> bytes:
        out = bytearray(P1)
        self.L.blst_p1_mult(_buf(out), _buf(p), _buf(scalar), nbits)
        return bytes(out)

    def msm_window(self, points, scalars, n, nbits, window) -> bytes:
        pbuf, sbuf = _buf(bytearray(points)), _buf(bytearray(scalars))
        parr = (C.c_void_p * 2)(C.cast(pbuf, C.c_void_p), None)
        sarr = (C.c_void_p * 2)(C.cast(sbuf, C.c_void_p), None)
        scratch = (C.c_uint64 * ((192 << max(0, window - 1)) // 8 + 1))()
        ret = bytearray(P1)
        self.L.blst_p1s_mult_pippenger_window(_buf(ret), parr, n, sarr, nbits, scratch, window)
        return self.compress(bytes(ret))

    def domain(self, n) -> bytes:
        L = self.L.blst_fr_fft_domain_len(n)
        out = bytearray(FR * L)
        assert self.L.blst_fr_fft_domain_init(_buf(out), L, n)
        return bytes(out)

    def p1_fft(self, values, n, inverse):
        b = bytearray(values)
        ok = self.L.blst_p1_fft(_buf(b), n, inverse)
        return ok, bytes(b)

    def p1_fft_with_domain(self, values, n, domain, domain_len, inverse):
        b = bytearray(values)
        ok = self.L.blst_p1_fft_with_domain(_buf(b), n, _buf(domain), domain_len, inverse)
        return ok, bytes(b)

    def p1_ifft_unscaled_with_domain(self, values, n, domain, domain_len):
        b = bytearray(values)
        ok = self.L.blst_p1_ifft_unscaled_with_domain(_buf(b), n, _buf(domain), domain_len)
        return ok, bytes(b)

    def p1_fft_truncated_prefix(self, values, n, xn, domain, domain_len):
        """The reference's fft_forward_truncated_prefix template (through
        oracle/ref_shim.cpp) over the domain's first n roots."""
        assert domain_len == n + 2 and 0 < xn <= n
        b = bytearray(values)
        ok = self.L.refshim_p1_fft_truncated_prefix(_buf(b), n, xn, _buf(domain))
        return ok, bytes(b)

    def fr_fft(self, values, n, inverse):
        b = bytearray(values)
        ok = self.L.blst_fr_fft(_buf(b), n, inverse)
        return ok, bytes(b)

    def fr_fft_with_domain(self, values, n, domain, domain_len, inverse):
        b = bytearray(values)
        ok = self.L.blst_fr_fft_with_domain(_buf(b), n, _buf(domain), domain_len, inverse)
        return ok, bytes(b)

    def uncompress(self, enc48: bytes, init: bytes = bytes(96)):
        out = bytearray(init)
        err = self.L.blst_p1_uncompress(_buf(out), _buf(enc48))
        return err, bytes(out)

    def deserialize(self, enc96: bytes, init: bytes = bytes(96)):
        out = bytearray(init)
        err = self.L.blst_p1_deserialize(_buf(out), _buf(enc96))
        return err, bytes(out)

    def in_g1(self, aff: bytes) -> bool:
        return bool(self.L.blst_p1_affine_in_g1(_buf(aff)))

    def msm_fr(self, points: bytes, frs: bytes, n: int) -> bytes:
        sz = self.L.blst_p1s_mult_pippenger_fr_scratch_sizeof(n)
        scratch = (C.c_uint64 * (sz // 8 + 1))()
        ret = bytearray(P1)
        ok = self.L.blst_p1s_mult_pippenger_fr(_buf(ret), _buf(points), _buf(frs), n, scratch, sz)
        assert ok
        return self.compress(bytes(ret))

    def mult_fr(self, points: bytes, frs: bytes, n: int) -> bytes:
        """blst_p1s_mult_fr (policy MSM) -> compressed."""
        size = self.L.blst_p1s_mult_fr_scratch_sizeof(n)
        scratch = (C.c_uint64 * (size // 8 + 1))()
        ret = bytearray(P1)
        assert self.L.blst_p1s_mult_fr(_buf(ret), _buf(bytearray(points)), _buf(bytearray(frs)), n, scratch, size)
        return self.compress(bytes(ret))

    def batch_affine_fr(self, points: bytes, frs: bytes, n: int, window: int, batch: int) -> bytes:
        """blst_p1s_mult_batch_affine_fr -> compressed."""
        size = self.L.blst_p1s_mult_batch_affine_fr_scratch_sizeof(n, window, batch)
        scratch = (C.c_uint64 * (size // 8 + 1))()
        ret = bytearray(P1)
        assert self.L.blst_p1s_mult_batch_affine_fr(_buf(ret), _buf(bytearray(points)), _buf(bytearray(frs)), n,
                                                    scratch, size, window, batch)
        return self.compress(bytes(ret))


def reference_available():
    return os.path.exists(REF_SO)
