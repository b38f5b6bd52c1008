"""Python mirror of the library's C ABI (ctypes over libcatmsm_gpu.so).

Function names, argument meaning and failure behaviour follow the reference's
C entry points (bindings/blst_scalar.h:535-539, :603; bindings/blst_fft.h:52-131):
the MSM returns the point at infinity on invalid input, the FFT calls return
False and leave the values unchanged.  Buffers are ``bytes``/``bytearray`` in
the reference ABI layouts (96-byte affine points, 144-byte Jacobian points,
32-byte scalars, 32-byte Montgomery Fr).

Loading fails loudly when the shared library is missing or cannot be built:
there is no CPU fallback.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcatmsm_gpu.so")

P1 = 144
P1A = 96
FR = 32

_vp = C.c_void_p
_sz = C.c_size_t

_lib = None


def load(build_if_missing=True):
    """Load (building first if needed) the CUDA library; raises on failure."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        import importlib.util
        spec = importlib.util.spec_from_file_location("catmsm_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libcatmsm_gpu.so is missing; run build.py")
    L = C.CDLL(LIB_PATH)
    L.blst_p1s_mult_pippenger_scratch_sizeof.restype = _sz
    L.blst_p1s_mult_pippenger_scratch_sizeof.argtypes = [_sz]
    L.blst_p1s_mult_pippenger_window_scratch_sizeof.restype = _sz
    L.blst_p1s_mult_pippenger_window_scratch_sizeof.argtypes = [_sz]
    L.blst_p1s_mult_pippenger.restype = None
    L.blst_p1s_mult_pippenger.argtypes = [_vp, _vp, _sz, _vp, _sz, _vp]
    L.blst_p1s_mult_pippenger_window.restype = None
    L.blst_p1s_mult_pippenger_window.argtypes = [_vp, _vp, _sz, _vp, _sz, _vp, _sz]
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
    L.catmsm_p1s_mult_pippenger_device.restype = C.c_int
    L.catmsm_p1s_mult_pippenger_device.argtypes = [_vp, _vp, _vp, _sz, _sz, _sz, _sz]
    L.catmsm_p1_fft_device.restype = C.c_int
    L.catmsm_p1_fft_device.argtypes = [_vp, _sz, _vp, C.c_int]
    L.blst_p1s_mult_pippenger_fr_scratch_sizeof.restype = _sz
    L.blst_p1s_mult_pippenger_fr_scratch_sizeof.argtypes = [_sz]
    L.blst_p1s_mult_pippenger_fr.restype = C.c_bool
    L.blst_p1s_mult_pippenger_fr.argtypes = [_vp, _vp, _vp, _sz, _vp, _sz]
    L.blst_fr_fft.restype = C.c_bool
    L.blst_fr_fft.argtypes = [_vp, _sz, C.c_bool]
    L.blst_fr_fft_with_domain.restype = C.c_bool
    L.blst_fr_fft_with_domain.argtypes = [_vp, _sz, _vp, _sz, C.c_bool]
    for f in ("catmsm_p1s_uncompress", "catmsm_p1s_deserialize"):
        getattr(L, f).restype = C.c_int
        getattr(L, f).argtypes = [_vp, _vp, _sz, _vp, C.c_int]
    L.catmsm_p1s_affine_in_g1.restype = C.c_int
    L.catmsm_p1s_affine_in_g1.argtypes = [_vp, _sz, _vp]
    L.catmsm_p1_fft_batch.restype = C.c_int
    L.catmsm_p1_fft_truncated_prefix.restype = C.c_bool
    L.catmsm_p1_fft_truncated_prefix.argtypes = [_vp, _sz, _sz, _vp, _sz]
    L.catmsm_p1_fft_batch.argtypes = [_vp, _vp, _vp, _vp, _sz]
    L.catmsm_stream.restype = _vp
    L.catmsm_stream.argtypes = []
    L.catmsm_launch_count.restype = C.c_long
    L.catmsm_launch_count.argtypes = []
    L.catmsm_msm_window.restype = _sz
    L.catmsm_msm_window.argtypes = [_sz]
    L.catmsm_msm_plan.restype = C.c_int
    L.catmsm_msm_plan.argtypes = [_sz, _sz, _vp, _vp, _vp]
    L.catmsm_msm_plan_detail.restype = C.c_int
    L.catmsm_msm_plan_detail.argtypes = [_sz, _sz, C.c_int, _vp, _vp, _vp, _vp, _vp]
    L.catmsm_msm_glv.restype = C.c_int
    L.catmsm_msm_glv.argtypes = [C.c_int]
    L.catmsm_msm_affine_rounds.restype = C.c_int
    L.catmsm_msm_affine_rounds.argtypes = [C.c_int]
    L.catmsm_msm_affine_rounds_for.restype = C.c_int
    L.catmsm_msm_affine_rounds_for.argtypes = [_sz, _sz]
    L.catmsm_fp_inv.restype = C.c_int
    L.catmsm_fp_inv.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
    L.catmsm_p1_affines_from_scalars.restype = C.c_int
    L.catmsm_p1_affines_from_scalars.argtypes = [_vp, _vp, _sz]
    L.catmsm_p1_affines_from_scalars_device.restype = C.c_int
    L.catmsm_p1_affines_from_scalars_device.argtypes = [_vp, _vp, _sz]
    L.catmsm_fp_mul.restype = C.c_int
    L.catmsm_fp_mul.argtypes = [_vp, _vp, _vp, _sz]
    L.catmsm_imad_peak.restype = C.c_double
    L.catmsm_imad_peak.argtypes = []
    L.catmsm_imad_peak_form.restype = C.c_double
    L.catmsm_imad_peak_form.argtypes = [C.c_int]
    L.catmsm_profile.restype = None
    L.catmsm_profile.argtypes = [C.c_int]
    L.catmsm_profile_reset.restype = None
    L.catmsm_profile_reset.argtypes = []
    L.catmsm_basis_create.restype = C.c_void_p
    L.catmsm_basis_create.argtypes = [_vp, _sz, _sz]
    L.catmsm_basis_destroy.restype = None
    L.catmsm_basis_destroy.argtypes = [_vp]
    L.catmsm_basis_config.restype = C.c_int
    L.catmsm_basis_config.argtypes = [_vp, _vp, _vp]
    L.catmsm_basis_set_config.restype = C.c_int
    L.catmsm_basis_set_config.argtypes = [_vp, _sz, _sz]
    L.catmsm_basis_msm_batch.restype = C.c_int
    L.catmsm_basis_msm_batch.argtypes = [_vp, _vp, _sz, _vp, _vp, C.c_int]
    L.catmsm_basis_autotune.restype = C.c_int
    L.catmsm_basis_autotune.argtypes = [_vp, _sz, _vp, _vp, C.c_int]
    L.catmsm_server_create.restype = C.c_void_p
    L.catmsm_server_create.argtypes = [_vp, _sz, _sz]
    L.catmsm_server_destroy.restype = None
    L.catmsm_server_destroy.argtypes = [_vp]
    L.catmsm_server_submit_msm.restype = C.c_int64
    L.catmsm_server_submit_msm.argtypes = [_vp, _vp, _sz]
    L.catmsm_server_submit_fft.restype = C.c_int64
    L.catmsm_server_submit_fft.argtypes = [_vp, _vp, _sz, _vp, C.c_int]
    L.catmsm_server_wait.restype = C.c_int
    L.catmsm_server_wait.argtypes = [_vp, C.c_int64, _vp, _vp]
    L.catmsm_server_stats.restype = C.c_int
    L.catmsm_server_stats.argtypes = [_vp, _vp, _vp, _vp, _vp]
    L.catmsm_profile_entries.restype = C.c_double
    L.catmsm_profile_entries.argtypes = []
    L.catmsm_profile_read.restype = C.c_int
    L.catmsm_profile_read.argtypes = [_vp, C.c_int, _vp]
    L.blst_p1s_mult_fr_scratch_sizeof.restype = _sz
    L.blst_p1s_mult_fr_scratch_sizeof.argtypes = [_sz]
    L.blst_p1s_mult_fr.restype = C.c_bool
    L.blst_p1s_mult_fr.argtypes = [_vp, _vp, _vp, _sz, _vp, _sz]
    L.blst_p1s_mult_batch_affine_fr_scratch_sizeof.restype = _sz
    L.blst_p1s_mult_batch_affine_fr_scratch_sizeof.argtypes = [_sz, _sz, _sz]
    L.blst_p1s_mult_batch_affine_fr.restype = C.c_bool
    L.blst_p1s_mult_batch_affine_fr.argtypes = [_vp, _vp, _vp, _sz, _vp, _sz, _sz, _sz]
    L.blst_p1s_tile_pippenger.restype = None
    L.blst_p1s_tile_pippenger.argtypes = [_vp, _vp, _sz, _vp, _sz, _vp, _sz, _sz]
    L.blst_p1s_mult_wbits_precompute_sizeof.restype = _sz
    L.blst_p1s_mult_wbits_precompute_sizeof.argtypes = [_sz, _sz]
    L.blst_p1s_mult_wbits_precompute.restype = None
    L.blst_p1s_mult_wbits_precompute.argtypes = [_vp, _sz, _vp, _sz]
    L.blst_p1s_mult_wbits_scratch_sizeof.restype = _sz
    L.blst_p1s_mult_wbits_scratch_sizeof.argtypes = [_sz]
    L.blst_p1s_mult_wbits.restype = None
    L.blst_p1s_mult_wbits.argtypes = [_vp, _vp, _sz, _sz, _vp, _sz, _vp]
    _lib = L
    return L


def _buf(data):
    if isinstance(data, bytearray):
        return (C.c_char * len(data)).from_buffer(data)
    return C.c_char_p(bytes(data))


def _addr(b):
    return C.cast(b, C.c_void_p)


def p1s_mult_pippenger(points: bytes, scalars: bytes, npoints: int, nbits: int = 255,
                       scratch: bool = True) -> bytes:
    """Contiguous-descriptor MSM through the C ABI; returns the 144-byte blst_p1."""
    L = load()
    pb = _buf(bytearray(points) if points else bytearray(96))
    sb = _buf(bytearray(scalars) if scalars else bytearray(32))
    parr = (C.c_void_p * 2)(_addr(pb), None)
    sarr = (C.c_void_p * 2)(_addr(sb), None)
    scr = (C.c_uint64 * 4)() if scratch else None
    ret = bytearray(P1)
    L.blst_p1s_mult_pippenger(_buf(ret), parr, npoints, sarr, nbits, scr)
    return bytes(ret)


def p1s_mult_pippenger_descriptors(point_ptrs, scalar_ptrs, npoints, nbits, scratch=True, window=None) -> bytes:
    """MSM with caller-built descriptor arrays (lists of addresses or None)."""
    L = load()
    parr = (C.c_void_p * len(point_ptrs))(*point_ptrs)
    sarr = (C.c_void_p * len(scalar_ptrs))(*scalar_ptrs)
    scr = (C.c_uint64 * 4)() if scratch else None
    ret = bytearray(P1)
    if window is None:
        L.blst_p1s_mult_pippenger(_buf(ret), parr, npoints, sarr, nbits, scr)
    else:
        L.blst_p1s_mult_pippenger_window(_buf(ret), parr, npoints, sarr, nbits, scr, window)
    return bytes(ret)


def p1s_mult_wbits_precompute_sizeof(wbits: int, n: int) -> int:
    return load().blst_p1s_mult_wbits_precompute_sizeof(wbits, n)


def p1s_mult_wbits_scratch_sizeof(n: int) -> int:
    return load().blst_p1s_mult_wbits_scratch_sizeof(n)


def p1s_mult_wbits_precompute(points: bytes, n: int, wbits: int, table: bytearray = None,
                              point_ptrs=None) -> bytes:
    """Fixed-base table of n rows of 2^(wbits-1) affine multiples.  `table`
    (optional) is the caller's buffer, written in place; `point_ptrs` an
    optional explicit descriptor array (addresses or None) instead of the
    contiguous `points`."""
    L = load()
    if table is None:
        table = bytearray(max(96, L.blst_p1s_mult_wbits_precompute_sizeof(wbits, n)))
    tb = _buf(table)
    if point_ptrs is None:
        pb = _buf(bytearray(points) if points else bytearray(96))
        point_ptrs = [C.cast(pb, C.c_void_p).value, None]
    parr = (C.c_void_p * len(point_ptrs))(*point_ptrs)
    L.blst_p1s_mult_wbits_precompute(tb, wbits, parr, n)
    return bytes(table)


def p1s_mult_wbits(table: bytes, wbits: int, n: int, scalars: bytes, nbits: int = 255,
                   scratch: bool = True, scalar_ptrs=None) -> bytes:
    """Fixed-table MSM through the C ABI; returns the 144-byte blst_p1."""
    L = load()
    tb = _buf(bytearray(table) if table else bytearray(96))
    if scalar_ptrs is None:
        sb = _buf(bytearray(scalars) if scalars else bytearray(32))
        scalar_ptrs = [C.cast(sb, C.c_void_p).value, None]
    sarr = (C.c_void_p * len(scalar_ptrs))(*scalar_ptrs)
    scr = (C.c_uint64 * 4)() if scratch else None
    ret = bytearray(P1)
    L.blst_p1s_mult_wbits(_buf(ret), tb if table is not None else None, wbits, n, sarr, nbits, scr)
    return bytes(ret)


def p1s_tile_pippenger(points: bytes, scalars: bytes, npoints: int, nbits: int, bit0: int, window: int,
                       scratch: bool = True) -> bytes:
    """One signed window of the MSM (blst_p1s_tile_pippenger); 144-byte blst_p1."""
    L = load()
    pb = _buf(bytearray(points) if points else bytearray(96))
    sb = _buf(bytearray(scalars) if scalars else bytearray(32))
    parr = (C.c_void_p * 2)(_addr(pb), None)
    sarr = (C.c_void_p * 2)(_addr(sb), None)
    scr = (C.c_uint64 * 4)() if scratch else None
    ret = bytearray(P1)
    L.blst_p1s_tile_pippenger(_buf(ret), parr, npoints, sarr, nbits, scr, bit0, window)
    return bytes(ret)


def scratch_sizeof(n: int) -> int:
    return load().blst_p1s_mult_pippenger_scratch_sizeof(n)


def window_scratch_sizeof(w: int) -> int:
    return load().blst_p1s_mult_pippenger_window_scratch_sizeof(w)


def fr_fft_domain_len(n: int) -> int:
    return load().blst_fr_fft_domain_len(n)


def fr_fft_domain_init(n: int, domain_len: int = None):
    L = load()
    dl = L.blst_fr_fft_domain_len(n) if domain_len is None else domain_len
    out = bytearray(FR * max(dl, 1))
    ok = L.blst_fr_fft_domain_init(_buf(out), dl, n)
    return ok, bytes(out)


def p1_fft(values: bytes, n: int, inverse: bool):
    b = bytearray(values)
    ok = load().blst_p1_fft(_buf(b) if b else None, n, inverse)
    return ok, bytes(b)


def p1_fft_with_domain(values: bytes, n: int, domain: bytes, domain_len: int, inverse: bool):
    b = bytearray(values)
    ok = load().blst_p1_fft_with_domain(_buf(b) if b else None, n, _buf(domain) if domain else None,
                                        domain_len, inverse)
    return ok, bytes(b)


def p1_ifft_unscaled_with_domain(values: bytes, n: int, domain: bytes, domain_len: int):
    b = bytearray(values)
    ok = load().blst_p1_ifft_unscaled_with_domain(_buf(b) if b else None, n, _buf(domain) if domain else None,
                                                  domain_len)
    return ok, bytes(b)


def p1_fft_truncated_prefix(values: bytes, n: int, xn: int, domain: bytes, domain_len: int):
    """Forward G1 FFT of values whose elements [xn, n) are the identity
    (the reference's fft_forward_truncated_prefix); returns (ok, values)."""
    b = bytearray(values)
    ok = load().catmsm_p1_fft_truncated_prefix(_buf(b) if b else None, n, xn, _buf(domain) if domain else None,
                                               domain_len)
    return ok, bytes(b)


def p1s_mult_pippenger_fr(points: bytes, frs: bytes, n: int, scratch_size=None, ret_init=None):
    """blst_p1s_mult_pippenger_fr; returns (ok, 144-byte ret)."""
    L = load()
    need = L.blst_p1s_mult_pippenger_fr_scratch_sizeof(n)
    size = need if scratch_size is None else scratch_size
    scratch = (C.c_uint64 * (max(size, 8) // 8 + 1))() if size >= 0 else None
    ret = bytearray(ret_init if ret_init is not None else bytes(P1))
    ok = L.blst_p1s_mult_pippenger_fr(_buf(ret), _buf(bytearray(points)) if points else None,
                                      _buf(bytearray(frs)) if frs else None, n, scratch, size if size >= 0 else 0)
    return ok, bytes(ret)


def p1s_mult_pippenger_fr_scratch_sizeof(n: int) -> int:
    return load().blst_p1s_mult_pippenger_fr_scratch_sizeof(n)


def p1s_mult_fr(points: bytes, frs: bytes, n: int, scratch_size=None, ret_init=None):
    """blst_p1s_mult_fr; returns (ok, 144-byte ret)."""
    L = load()
    size = L.blst_p1s_mult_fr_scratch_sizeof(n) if scratch_size is None else scratch_size
    scratch = (C.c_uint64 * (max(size, 8) // 8 + 1))() if size >= 0 else None
    ret = bytearray(ret_init if ret_init is not None else bytes(P1))
    ok = L.blst_p1s_mult_fr(_buf(ret), _buf(bytearray(points)) if points else None,
                            _buf(bytearray(frs)) if frs else None, n, scratch, size if size >= 0 else 0)
    return ok, bytes(ret)


def p1s_mult_fr_scratch_sizeof(n: int) -> int:
    return load().blst_p1s_mult_fr_scratch_sizeof(n)


def p1s_mult_batch_affine_fr(points: bytes, frs: bytes, n: int, window: int, batch_size: int,
                             scratch_size=None, ret_init=None):
    """blst_p1s_mult_batch_affine_fr; returns (ok, 144-byte ret)."""
    L = load()
    need = L.blst_p1s_mult_batch_affine_fr_scratch_sizeof(n, window, batch_size)
    size = need if scratch_size is None else scratch_size
    scratch = (C.c_uint64 * (max(size, 8) // 8 + 1))() if size >= 0 else None
    ret = bytearray(ret_init if ret_init is not None else bytes(P1))
    ok = L.blst_p1s_mult_batch_affine_fr(_buf(ret), _buf(bytearray(points)) if points else None,
                                         _buf(bytearray(frs)) if frs else None, n, scratch,
                                         size if size >= 0 else 0, window, batch_size)
    return ok, bytes(ret)


def p1s_mult_batch_affine_fr_scratch_sizeof(n: int, window: int, batch_size: int) -> int:
    return load().blst_p1s_mult_batch_affine_fr_scratch_sizeof(n, window, batch_size)


def fr_fft(values: bytes, n: int, inverse: bool):
    b = bytearray(values)
    ok = load().blst_fr_fft(_buf(b) if b else None, n, inverse)
    return ok, bytes(b)


def fr_fft_with_domain(values: bytes, n: int, domain: bytes, domain_len: int, inverse: bool):
    b = bytearray(values)
    ok = load().blst_fr_fft_with_domain(_buf(b) if b else None, n, _buf(domain) if domain else None,
                                        domain_len, inverse)
    return ok, bytes(b)


def p1s_decode(encodings: bytes, n: int, compressed: bool, init: bytes = None, check_group=False):
    """Batch uncompress (48-byte) / deserialize (96-byte) elements; returns
    (rc, list of BLST_ERROR codes, affine outputs bytes)."""
    L = load()
    out = bytearray(init if init is not None else bytes(96 * n))
    errs = (C.c_int * max(n, 1))()
    f = L.catmsm_p1s_uncompress if compressed else L.catmsm_p1s_deserialize
    rc = f(_buf(out), _buf(bytearray(encodings)), n, errs, 1 if check_group else 0)
    return rc, list(errs)[:n], bytes(out)


def p1s_affine_in_g1(points: bytes, n: int):
    L = load()
    res = (C.c_int * max(n, 1))()
    rc = L.catmsm_p1s_affine_in_g1(_buf(bytearray(points)), n, res)
    return rc, [bool(x) for x in list(res)[:n]]


def p1_fft_batch(values_list, ns, domains, modes):
    """Batch of G1 FFTs; returns (rc, list of output byte strings)."""
    bufs = [bytearray(v) for v in values_list]
    rc = p1_fft_batch_inplace(bufs, ns, domains, modes)
    return rc, [bytes(b) for b in bufs]


def p1_fft_batch_inplace(bufs, ns, domains, modes):
    """Batch of G1 FFTs transforming the given bytearrays in place (domains:
    bytes or bytearray, read only); returns the status code."""
    L = load()
    vb = [(C.c_char * len(b)).from_buffer(b) for b in bufs]
    db = [(C.c_char * len(d)).from_buffer(d) if isinstance(d, bytearray) else C.c_char_p(bytes(d)) for d in domains]
    count = len(bufs)
    varr = (C.c_void_p * count)(*[C.cast(x, C.c_void_p) for x in vb])
    darr = (C.c_void_p * count)(*[C.cast(x, C.c_void_p) for x in db])
    narr = (C.c_size_t * count)(*ns)
    marr = (C.c_int * count)(*modes)
    return L.catmsm_p1_fft_batch(varr, narr, darr, marr, count)


def points_from_scalars(k32: bytes, n: int) -> bytes:
    out = bytearray(P1A * n)
    rc = load().catmsm_p1_affines_from_scalars(_buf(out), _buf(k32), n)
    if rc != 0:
        raise RuntimeError("catmsm_p1_affines_from_scalars failed: %d" % rc)
    return bytes(out)


def fp_mul(a: bytes, b: bytes, n: int) -> bytes:
    out = bytearray(48 * n)
    rc = load().catmsm_fp_mul(_buf(out), _buf(a), _buf(b), n)
    if rc != 0:
        raise RuntimeError("catmsm_fp_mul failed: %d" % rc)
    return bytes(out)


def msm_device(d_points: int, d_scalars: int, stride: int, n: int, nbits: int, window: int = 0) -> bytes:
    ret = bytearray(P1)
    rc = load().catmsm_p1s_mult_pippenger_device(_buf(ret), d_points, d_scalars, stride, n, nbits, window)
    if rc != 0:
        raise RuntimeError("catmsm_p1s_mult_pippenger_device failed: %d" % rc)
    return bytes(ret)


def fft_device(d_values: int, n: int, d_domain: int, mode: int) -> None:
    rc = load().catmsm_p1_fft_device(d_values, n, d_domain, mode)
    if rc != 0:
        raise RuntimeError("catmsm_p1_fft_device failed: %d" % rc)


def stream_handle() -> int:
    return load().catmsm_stream()


def launch_count() -> int:
    return load().catmsm_launch_count()


def msm_window(n: int) -> int:
    return load().catmsm_msm_window(n)


STAGES = ("prep", "digits", "scan", "scatter", "accumulate", "fixup", "reduce", "host_fold")


def msm_plan(n: int, nbits: int = 255):
    """(window, windows, pipeline points) of this thread's next MSM."""
    c, d, p = _sz(), _sz(), _sz()
    assert load().catmsm_msm_plan(n, nbits, C.byref(c), C.byref(d), C.byref(p)) == 0
    return c.value, d.value, p.value


def msm_plan_detail(n: int, nbits: int = 255, glv: int = 1):
    """(window, windows, pipeline points, chunk length, level-1 fan-in) of an
    MSM; host arithmetic only, no GPU needed."""
    v = [_sz() for _ in range(5)]
    assert load().catmsm_msm_plan_detail(n, nbits, glv, *[C.byref(x) for x in v]) == 0
    return tuple(x.value for x in v)


def msm_glv(enable: int = -1) -> int:
    """Set (0/1) or query (-1) the GLV split for this thread; returns the previous setting."""
    return load().catmsm_msm_glv(enable)


def msm_affine_rounds(rounds: int = -2) -> int:
    """Set (-1 = by size, 0..8) or query (-2) this thread's batch-affine
    accumulation rounds; returns the previous setting."""
    return load().catmsm_msm_affine_rounds(rounds)


def msm_affine_rounds_for(n: int, nbits: int = 255) -> int:
    """Batch-affine rounds this thread's next MSM of n points would run."""
    return load().catmsm_msm_affine_rounds_for(n, nbits)


def fp_inv(a: bytes, n: int) -> bytes:
    """Montgomery-form inverses of n field elements (0 -> 0) on the device
    (the variable-time inversion of the batch-affine rounds)."""
    out = bytearray(48 * n)
    rc = load().catmsm_fp_inv(_buf(out), _buf(a), n)
    if rc != 0:
        raise RuntimeError("catmsm_fp_inv failed: %d" % rc)
    return bytes(out)


def imad_peak_tera() -> float:
    """Measured device IMAD throughput, tera-IMAD/s."""
    return load().catmsm_imad_peak()


def imad_peak_forms():
    """(mad.lo, mad.wide) measured tera-IMAD/s."""
    L = load()
    return L.catmsm_imad_peak_form(0), L.catmsm_imad_peak_form(1)


def profile(enable: bool) -> None:
    load().catmsm_profile(1 if enable else 0)


def profile_reset() -> None:
    load().catmsm_profile_reset()


def profile_read():
    """{stage: accumulated ms}, number of profiled calls."""
    ms = (C.c_double * len(STAGES))()
    calls = C.c_long(0)
    load().catmsm_profile_read(ms, len(STAGES), C.byref(calls))
    return dict(zip(STAGES, list(ms))), calls.value


def profile_entries() -> float:
    return load().catmsm_profile_entries()


class Basis:
    """A resident basis with fixed-base tables for batched commitments
    (catmsm_basis_*; no reference counterpart)."""

    def __init__(self, points: bytes, n: int, window: int = 0):
        self.L = load()
        self.n = n
        self._pts = bytearray(points)
        self.h = self.L.catmsm_basis_create(_buf(self._pts), n, window)
        if not self.h:
            raise RuntimeError("catmsm_basis_create failed")

    def close(self):
        if self.h:
            self.L.catmsm_basis_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def config(self):
        w, c = C.c_size_t(), C.c_size_t()
        self.L.catmsm_basis_config(self.h, C.byref(w), C.byref(c))
        return w.value, c.value

    def set_config(self, window, chunk):
        rc = self.L.catmsm_basis_set_config(self.h, window, chunk)
        if rc != 0:
            raise RuntimeError("catmsm_basis_set_config failed: %d" % rc)

    def _args(self, counts, scalars):
        """counts as a size_t array; scalars as a pointer without copying:
        bytes / bytearray (read in place) or an int host address (e.g. a
        pinned buffer's data_ptr())."""
        cnt = (C.c_size_t * len(counts))(*counts)
        if isinstance(scalars, int):
            return cnt, C.c_void_p(scalars)
        if isinstance(scalars, bytearray):
            return cnt, (C.c_char * len(scalars)).from_buffer(scalars)
        return cnt, C.c_char_p(bytes(scalars))

    def msm_batch(self, counts, scalars: bytes, use_graph=True) -> bytes:
        """counts[j] points per MSM; scalars: concatenated 32-byte scalars.
        Returns len(counts) Jacobian blst_p1 (144 bytes each)."""
        cnt, sb = self._args(counts, scalars)
        out = bytearray(P1 * len(counts))
        rc = self.L.catmsm_basis_msm_batch(self.h, _buf(out), len(counts), cnt, sb, 1 if use_graph else 0)
        if rc != 0:
            raise RuntimeError("catmsm_basis_msm_batch failed: %d" % rc)
        return bytes(out)

    def autotune(self, counts, scalars: bytes, force=False):
        cnt, sb = self._args(counts, scalars)
        rc = self.L.catmsm_basis_autotune(self.h, len(counts), cnt, sb, 1 if force else 0)
        if rc != 0:
            raise RuntimeError("catmsm_basis_autotune failed: %d" % rc)
        return self.config()


class Server:
    """Continuous-batching request engine over a resident Basis
    (catmsm_server_*; no reference counterpart).  Submitted buffers are kept
    alive here until their ticket is waited on."""

    def __init__(self, basis: "Basis", workers: int = 4, hbm_budget: int = 0):
        self.L = load()
        self.basis = basis
        self.h = self.L.catmsm_server_create(basis.h, workers, hbm_budget)
        if not self.h:
            raise RuntimeError("catmsm_server_create failed")
        self._keep = {}

    def close(self):
        if self.h:
            self.L.catmsm_server_destroy(self.h)
            self.h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit_msm(self, scalars: bytes, k: int) -> int:
        buf = (C.c_char * len(scalars)).from_buffer_copy(scalars)
        t = self.L.catmsm_server_submit_msm(self.h, buf, k)
        if t < 0:
            raise ValueError("submit_msm rejected")
        self._keep[t] = (buf,)
        return t

    def submit_msm_ptr(self, addr: int, k: int) -> int:
        """MSM request whose k scalars live at host address `addr` (no copy;
        the caller keeps that memory alive until wait returns)."""
        t = self.L.catmsm_server_submit_msm(self.h, addr, k)
        if t < 0:
            raise ValueError("submit_msm rejected")
        self._keep[t] = ()
        return t

    def submit_fft(self, values: bytes, n: int, domain: bytes, mode: int) -> int:
        vb = (C.c_char * len(values)).from_buffer_copy(values)
        db = (C.c_char * len(domain)).from_buffer_copy(domain)
        t = self.L.catmsm_server_submit_fft(self.h, vb, n, db, mode)
        if t < 0:
            raise ValueError("submit_fft rejected")
        self._keep[t] = (vb, db)
        return t

    def wait(self, ticket: int):
        """(status, result bytes (MSM: 144-B Jacobian; FFT: the values), queue_ms, latency_ms)."""
        out = (C.c_char * P1)()
        times = (C.c_double * 2)()
        rc = self.L.catmsm_server_wait(self.h, ticket, out, times)
        keep = self._keep.pop(ticket)
        res = bytes(keep[0]) if len(keep) == 2 else bytes(out)
        return rc, res, times[0], times[1]

    def stats(self):
        a, b, c, d = C.c_long(), C.c_long(), C.c_long(), C.c_long()
        self.L.catmsm_server_stats(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d))
        return {"batches": a.value, "requests": b.value, "max_batch": c.value, "max_concurrent": d.value}
