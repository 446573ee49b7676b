"""Output files of the photon-transport path, in the reference's formats.

* ``.mch`` -- detected photons: the 64-byte History header
  (src/mcx_utils.h:113-130), then ``savedphoton`` records of ``colcount``
  float32, then the RNG seeds (``seedbyte`` bytes each), as
  mcx_savedetphoton writes them (src/mcx_utils.c:963-998).
* ``_detp.jdat`` -- detected photons in JData JSON (src/mcx_utils.c:1010-1190):
  ``MCXData.Info`` (the header values and the media), ``MCXData.PhotonData``
  with one array per record column group (detid, nscat, ppath, mom, p, v, w0)
  and the seeds.
* ``.jnii`` -- a volume (fluence etc.) in JNIfTI JSON (src/mcx_utils.c:761-884):
  ``NIFTIHeader`` and ``NIFTIData``.

Arrays use the JData annotation (``_ArrayType_``, ``_ArraySize_``,
``_ArrayZipType_``, ``_ArrayZipSize_``, ``_ArrayZipData_``: zlib-compressed,
base64-encoded little-endian bytes), as mcx_jdataencode does
(src/mcx_utils.c:4396-4470).
"""
import base64
import json
import struct
import zlib

import numpy as np

# History header (src/mcx_utils.h:113-130): magic, 7 uint32, float, uint32,
# float, int32, 3 uint32, 1 reserved int32 -> 64 bytes
_HDR = struct.Struct("<4s7IfIfi3Ii")
HEADER_FIELDS = ("magic", "version", "maxmedia", "detnum", "colcount", "totalphoton", "detected", "savedphoton",
                 "unitinmm", "seedbyte", "normalizer", "respin", "srcnum", "savedetflag", "totalsource", "reserved")
_DTYPES = {"single": np.float32, "double": np.float64, "uint32": np.uint32, "int32": np.int32, "uint8": np.uint8,
           "int8": np.int8, "uint16": np.uint16, "int16": np.int16, "uint64": np.uint64, "int64": np.int64}
# savedetflag bit -> (name, columns per record, JData type), src/mcx_utils.c:1075-1077
_COLUMNS = [("detid", 1, "uint32"), ("nscat", None, "uint32"), ("ppath", None, "single"), ("mom", None, "single"),
            ("p", 3, "single"), ("v", 3, "single"), ("w0", 1, "single")]


def header(maxmedia, detnum, colcount, totalphoton, detected, savedphoton, unitinmm=1.0, seedbyte=0,
           normalizer=0.0, respin=1, srcnum=1, savedetflag=0x5, totalsource=1):
    """A History header dictionary (version 1, magic 'MCXH')."""
    return dict(magic=b"MCXH", version=1, maxmedia=maxmedia, detnum=detnum, colcount=colcount,
                totalphoton=totalphoton, detected=detected, savedphoton=savedphoton, unitinmm=unitinmm,
                seedbyte=seedbyte, normalizer=normalizer, respin=respin, srcnum=srcnum, savedetflag=savedetflag,
                totalsource=totalsource, reserved=0)


def save_mch(path, detp, hdr, seeds=None, append=False):
    """detp: [colcount, n] float32 (run()'s 'detp'); seeds: [seedbyte, n] uint8 or None."""
    detp = np.asarray(detp, np.float32)
    h = dict(hdr)
    if detp.shape[0] != h["colcount"]:
        raise ValueError("detp has %d rows, the header says %d columns" % (detp.shape[0], h["colcount"]))
    with open(path, "ab" if append else "wb") as f:
        f.write(_HDR.pack(*[h[k] for k in HEADER_FIELDS]))
        f.write(np.ascontiguousarray(detp.T).tobytes())
        if seeds is not None:
            f.write(np.ascontiguousarray(np.asarray(seeds, np.uint8).T).tobytes())


def load_mch(path):
    """Returns (detp [colcount, n], seeds [seedbyte, n] or None, header) of
    every block in the file, concatenated (a file may hold appended blocks)."""
    raw = open(path, "rb").read()
    pos, dets, seeds, hdr = 0, [], [], None
    while pos < len(raw):
        vals = _HDR.unpack_from(raw, pos)
        h = dict(zip(HEADER_FIELDS, vals))
        if h["magic"] != b"MCXH":
            raise ValueError("not an mch block at byte %d" % pos)
        pos += _HDR.size
        n, c = h["savedphoton"], h["colcount"]
        d = np.frombuffer(raw, np.float32, n * c, pos).reshape(n, c).T
        pos += 4 * n * c
        dets.append(d)
        if h["seedbyte"]:
            s = np.frombuffer(raw, np.uint8, n * h["seedbyte"], pos).reshape(n, h["seedbyte"]).T
            pos += n * h["seedbyte"]
            seeds.append(s)
        hdr = h if hdr is None else dict(hdr, savedphoton=hdr["savedphoton"] + n)
    detp = np.concatenate(dets, axis=1) if dets else np.zeros((0, 0), np.float32)
    return detp, (np.concatenate(seeds, axis=1) if seeds else None), hdr


def jdata_encode(arr, jtype, zipped=True, order=None):
    """An array as a JData annotated object (zlib + base64, or base64 only)."""
    a = np.ascontiguousarray(np.asarray(arr, _DTYPES[jtype]))
    raw = a.astype(a.dtype.newbyteorder("<"), copy=False).tobytes()
    obj = {"_ArrayType_": jtype, "_ArraySize_": list(a.shape)}
    if order:
        obj["_ArrayOrder_"] = order
    obj["_ArrayZipType_"] = "zlib" if zipped else "base64"
    obj["_ArrayZipSize_"] = int(a.size)
    obj["_ArrayZipData_"] = base64.b64encode(zlib.compress(raw) if zipped else raw).decode()
    return obj


def jdata_decode(obj):
    data = base64.b64decode(obj["_ArrayZipData_"])
    if obj.get("_ArrayZipType_", "zlib") == "zlib":
        data = zlib.decompress(data)
    a = np.frombuffer(data, np.dtype(_DTYPES[obj["_ArrayType_"]]).newbyteorder("<"))
    shape = obj["_ArraySize_"]
    if obj.get("_ArrayOrder_") == "c" and len(shape) > 1:
        return a.reshape(shape[::-1]).T.copy()
    return a.reshape(shape).copy()


def save_jdet(path, detp, hdr, prop, seeds=None, zipped=True):
    """Detected photons as JData JSON.  prop: medianum rows {mua, mus, g, n}
    in the run's length unit (mua and mus are divided by the header's
    unitinmm, as the reference writes them per mm).  Header floats are the
    float32 values the reference's header holds."""
    detp = np.asarray(detp, np.float32)
    h = dict(hdr)
    f32 = np.float32
    unit = f32(h["unitinmm"])
    info = {"Version": h["version"], "MediaNum": h["maxmedia"], "DetNum": h["detnum"], "ColumnNum": h["colcount"],
            "TotalPhoton": h["totalphoton"], "DetectedPhoton": int(detp.shape[1]), "SavedPhoton": h["savedphoton"],
            "LengthUnit": float(unit), "SeedByte": h["seedbyte"], "Normalizer": float(f32(h["normalizer"])),
            "Repeat": h["respin"], "SrcNum": h["srcnum"], "SaveDetFlag": h["savedetflag"],
            "TotalSource": h["totalsource"],
            "Media": [{"mua": float(r[0] / unit), "mus": float(r[1] / unit), "g": float(r[2]), "n": float(r[3])}
                      for r in np.asarray(prop, f32).reshape(-1, 4)]}
    data = {}
    col = 0
    n = detp.shape[1]
    for bit, (name, width, jtype) in enumerate(_COLUMNS):
        if not (h["savedetflag"] >> bit) & 1:
            continue
        w = h["maxmedia"] if width is None else width
        block = detp[col:col + w].T                # [n, w]
        if jtype == "uint32":
            vals = block.astype(np.int64).astype(np.uint32)
            if name == "detid" and h["totalsource"] > 1:
                data["srcid"] = jdata_encode((vals >> 16).reshape(n, w), "uint32", zipped)
                vals = vals & 0xFFFF
            data[name] = jdata_encode(vals.reshape(n, w), "uint32", zipped)
        else:
            data[name] = jdata_encode(block.reshape(n, w), "single", zipped)
        col += w
    if seeds is not None:
        data["seed"] = jdata_encode(np.asarray(seeds, np.uint8).T, "uint8", zipped)
    with open(path, "w") as f:
        json.dump({"MCXData": {"Info": info, "PhotonData": data}}, f, indent=1)
        f.write("\n")


def load_jdet(path):
    """Returns ({column group: array}, Info)."""
    d = json.load(open(path))["MCXData"]
    return {k: jdata_decode(v) for k, v in d["PhotonData"].items()}, d["Info"]


# NIFTIHeader.Description by output type (src/mcx_utils.c:814-819)
_JNII_DESCRIPTION = ["MCX volumetric output: Fluence rate (W/mm^2)", "MCX volumetric output: Fluence (J/mm^2)",
                     "MCX volumetric output: Voxel-wise energy deposit (J)",
                     "MCX volumetric output: Jacobian for mua (J/mm)", "MCX volumetric output: Scattering count",
                     "MCX volumetric output: Partial momentum transfer"]


def save_jnii(path, vol, voxelsize=(1.0, 1.0, 1.0), name="", outputtype=0, maxgate=1, zipped=True):
    """A volume ([Nx, Ny, Nz(, gates, ...)], x fastest as run() returns it) as
    JNIfTI JSON, with the header the reference writes (mcx_savejnii,
    src/mcx_utils.c:761-884): Name the session, LastSliceID the gate count,
    Description by output type (0 flux .. 5 momentum; -1 the generic one)."""
    v = np.asarray(vol, np.float32)
    dims = list(v.shape)
    vs = [float(np.float32(x)) for x in list(voxelsize) + [1.0] * (len(dims) - len(voxelsize))]
    desc = _JNII_DESCRIPTION[outputtype] if 0 <= outputtype < len(_JNII_DESCRIPTION) else "MCX volumetric output"
    hdr = {"NIIHeaderSize": 348, "Dim": dims, "Param1": 0, "Param2": 0, "Param3": 0, "Intent": 0,
           "DataType": "single", "BitDepth": 32, "FirstSliceID": 0, "VoxelSize": vs[:len(dims)],
           "Orientation": {"x": "r", "y": "a", "z": "s"}, "ScaleSlope": 1, "ScaleOffset": 0,
           "LastSliceID": int(maxgate), "SliceType": 1, "Unit": {"L": "mm", "T": "s"},
           "MaxIntensity": 1, "MinIntensity": 0, "SliceTime": 0, "TimeOffset": 0, "Description": desc,
           "AuxFile": "", "QForm": 0, "SForm": 1, "Quatern": {"b": 0, "c": 0, "d": 0},
           "QuaternOffset": {"x": 0, "y": 0, "z": 0}, "Affine": [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]],
           "Name": name, "NIIFormat": "jnifti"}
    # column-major (x fastest) data, marked with _ArrayOrder_ 'c' as the reference does
    data = jdata_encode(np.asfortranarray(v).ravel(order="F").reshape(dims[::-1]), "single", zipped, order="c")
    data["_ArraySize_"] = dims
    with open(path, "w") as f:
        json.dump({"_DataInfo_": {"JNIFTIVersion": "0.5", "Comment": "Created by mcxcl_gb300",
                                  "AnnotationFormat": "https://neurojson.org/jnifti/draft1",
                                  "SerialFormat": "https://json.org",
                                  "Parser": {"Python": ["https://neurojson.org/download/pyjdata",
                                                        "https://neurojson.org/download/pybjdata"],
                                             "MATLAB": ["https://neurojson.org/download/jnifty",
                                                        "https://neurojson.org/download/jsonlab"]}},
                   "NIFTIHeader": hdr, "NIFTIData": data}, f, indent=1)
        f.write("\n")


def load_jnii(path):
    d = json.load(open(path))
    return jdata_decode(d["NIFTIData"]), d["NIFTIHeader"]
