"""Volume encodings of the pmcxcl ``vol`` input (src/pmcxcl.cpp:93-426).

The array's dtype and leading dimension choose the media format; each voxel
becomes one 32-bit word (x fastest) that the transport kernel decodes
(updateproperty, src/mcx_core.cl:1079-1187):

| input | format | word |
|---|---|---|
| integer [Nx,Ny,Nz] | labels (1/2/4) | label |
| float32 [1,Nx,Ny,Nz] | MEDIA_MUA_FLOAT (101) | mua x unitinmm as float bits |
| float32 [2,Nx,Ny,Nz] | MEDIA_AS_F2H (100) | half(mua x unitinmm) \\| half(mus x unitinmm) << 16 |
| float32 [3,Nx,Ny,Nz] | MEDIA_LABEL_HALF (99) | label \\| property index << 14 \\| half(value) << 16 |
| uint8/int8 [4,Nx,Ny,Nz] | MEDIA_ASGN_BYTE (103) | four bytes: mua, mus, g, n between prop rows 1 and 2 |
| int16 [2,Nx,Ny,Nz] | MEDIA_AS_SHORT (104) | two shorts: mua, mus between prop rows 1 and 2 |
| uint8 [8,Nx,Ny,Nz] | MEDIA_2LABEL_SPLIT (97) | two planes: labels and plane point x y; point z and normal |
"""
import numpy as np

MEDIA_LABEL_HALF, MEDIA_AS_F2H, MEDIA_MUA_FLOAT, MEDIA_AS_HALF, MEDIA_ASGN_BYTE, MEDIA_AS_SHORT = 99, 100, 101, 102, 103, 104
MEDIA_2LABEL_SPLIT = 97
EPS = np.float32(1e-10)


def float_to_half_bits(x):
    """The reference's float -> half conversion (src/pmcxcl.cpp:300-325): the
    mantissa is truncated, exponents at or below 2^-15 take a denormal path
    when the top mantissa bits are small.  x: float32 array; returns uint16."""
    b = np.asarray(x, np.float32).view(np.uint32).astype(np.int64)
    m = (b >> 13) & 0x03FF
    e = (b >> 23) & 0xFF
    mask = np.where(e > 0x70, 0x1F, 0)
    tmp = ((e - 0x70) & mask) & 0xFFFF
    den = (m < 0x10) & (tmp == 0)
    # denormal branch
    sign = (b >> 16) & 0x8000
    md = ((b >> 12) & 0x07FF) | 0x0800
    s1 = 114 - e
    s2 = 113 - e
    h_den = sign | (np.where(s1 < 16, md >> np.clip(s1, 0, 63), 0) + (np.where(s2 < 16, md >> np.clip(s2, 0, 63), 0) & 1))
    # normal branch
    h_norm = ((((b >> 31) << 5) | tmp) << 10) | ((b >> 13) & 0x3FF)
    return (np.where(den, h_den, h_norm) & 0xFFFF).astype(np.uint16)


def encode(vol, unitinmm=1.0, alloc=None, native=True):
    """Returns (words uint32 [Nx*Ny*Nz], mediabyte, (Nx, Ny, Nz)).  alloc(n),
    when given, supplies the uint32 array a label volume is written into.
    native=False converts byte labels with numpy instead of the library's
    tiled transpose (same words)."""
    vol = np.asarray(vol)
    u = np.float32(unitinmm)
    if vol.ndim == 4:
        lead = vol.shape[0]
        dims = vol.shape[1:]
        # voxel-major with x fastest: [lead, Nx, Ny, Nz] in Fortran order
        comps = np.asfortranarray(vol).reshape(lead, -1, order="F")
        if vol.dtype == np.float32 and lead == 1:
            f = (comps[0] * u).astype(np.float32)
            w = f.view(np.uint32).copy()
            w[w == 0] = EPS.view(np.uint32)
            w[np.isnan(comps[0])] = 0
            return w, MEDIA_MUA_FLOAT, dims
        if vol.dtype == np.float32 and lead == 2:
            h0 = float_to_half_bits((comps[0] * u).astype(np.float32)).astype(np.uint32)
            h1 = float_to_half_bits((comps[1] * u).astype(np.float32)).astype(np.uint32)
            w = h0 | (h1 << 16)
            w[w == 0] = 0x00010000
            return w.astype(np.uint32), MEDIA_AS_F2H, dims
        if vol.dtype == np.float32 and lead == 3:
            val, kind, label = comps[0].astype(np.float32), comps[1], comps[2]
            if np.any((kind < 0) | (kind >= 4) | (label < 0)):
                raise ValueError("the 2nd volume must have an integer value between 0 and 3")
            val = np.where((kind >= 1) & (kind <= 2), (val * u).astype(np.float32), val).astype(np.float32)
            lo = (((kind.astype(np.uint8).astype(np.uint32) & 0x3) << 14) | label.astype(np.uint16).astype(np.uint32)) & 0xFFFF
            hi = np.zeros_like(lo)
            vb = val.view(np.uint32).astype(np.int64)
            e = (vb >> 23) & 0xFF
            tmp = ((e - 0x70) & np.where(e > 0x70, 0x1F, 0)) & 0xFFFF
            hi = (((((vb >> 31) << 5) | tmp) << 10) | ((vb >> 13) & 0x3FF)) & 0xFFFF
            return (lo | (hi.astype(np.uint32) << 16)).astype(np.uint32), MEDIA_LABEL_HALF, dims
        if vol.dtype in (np.uint8, np.int8) and lead == 4:
            b = np.ascontiguousarray(comps.T.astype(np.uint8))
            return b.view(np.uint32).reshape(-1).copy(), MEDIA_ASGN_BYTE, dims
        if vol.dtype in (np.int16, np.uint16) and lead == 2:
            s = np.ascontiguousarray(comps.T.astype(np.uint16))
            return s.view(np.uint32).reshape(-1).copy(), MEDIA_AS_SHORT, dims
        if vol.dtype in (np.int16, np.uint16) and lead == 3:
            raise ValueError("two-label mixture volumes (MEDIA_2LABEL_MIX) are not supported by this build")
        if vol.dtype in (np.uint8, np.int8) and lead == 8:
            # split voxels: bytes {lower label, upper label, reference point x y z, normal x y z}
            # (0..255 each) -> two planes, the labels and point x y first, point z and the
            # normal second (src/mcx_utils.c:1688-1711)
            b = comps.astype(np.uint8).astype(np.uint32)
            plane1 = b[3] | (b[2] << 8) | (b[1] << 16) | (b[0] << 24)
            plane2 = b[7] | (b[6] << 8) | (b[5] << 16) | (b[4] << 24)
            return np.concatenate([plane1, plane2]).astype(np.uint32), MEDIA_2LABEL_SPLIT, dims
        raise ValueError("unsupported 4-D volume: dtype %s with leading dimension %d" % (vol.dtype, lead))
    if vol.ndim == 2:
        vol = vol.reshape(vol.shape + (1,))
    if vol.ndim != 3:
        raise ValueError("the 'vol' field must be a 2-D or 3-D array of labels or a 4-D array of properties")
    if vol.dtype.kind not in "uifb":
        raise TypeError("unsupported volume dtype %s" % vol.dtype)
    words = alloc(vol.size) if alloc else np.empty(vol.size, np.uint32)
    if native and vol.dtype.itemsize == 1 and vol.dtype.kind in "ub" and \
            (vol.flags.c_contiguous or vol.flags.f_contiguous) and vol.size:
        # byte labels: the library's tiled transpose-and-widen, x fastest
        from . import _lib
        nx, ny, nz = (int(d) for d in vol.shape)
        _lib.load().mcx_labels_u8(vol.ctypes.data, nx, ny, nz, 0 if vol.flags.f_contiguous else 1,
                                  words.ctypes.data)
    else:
        # x fastest: one strided pass that transposes and widens
        words.reshape(vol.shape[::-1])[...] = vol.T
    mb = {1: 1, 2: 2}.get(vol.dtype.itemsize, 4) if vol.dtype.kind in "uib" else 4
    return words, mb, vol.shape
