"""Generate the committed golden fixtures from the reference's own test data.

Reads (in this container only) the reference testsuite's expected images
and text outputs and writes small fixtures next to this script:
  * noise-family and spline images (uint8 TIFF, Deflate) -> <name>.npz,
    subsampled;
  * testsuite/example-batched-deformer/ref/out.txt -> deformer_out.txt,
    testsuite/splineinverse/ref/out.txt -> splineinverse_out.txt and the
    closure print outputs of testsuite/closure, closure-zero and
    closure-conditional -> closure_*out.txt, testsuite/matrix and transform
    ref/out.txt -> matrix_out.txt, transform_out.txt;
  * src/liboslnoise/oslnoise_test.cpp known answers -> oslnoise_known.json.
The GPU machine never reads the reference; tests read only these fixtures.

Usage: python make_golden.py [REFERENCE_SOURCE_TREE]; the tree defaults to
$OSL_REFERENCE_ROOT, else /root/reference.

TIFF decoding is a minimal baseline-TIFF reader (strips, Deflate, LZW or no
compression, optional horizontal predictor) on top of zlib and numpy.
"""
import json
import os
import re
import struct
import sys
import zlib

import numpy as np

REF = os.environ.get("OSL_REFERENCE_ROOT", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))
STEP = 4  # keep every 4th pixel in x and y


def lzw_decode(data):
    """TIFF 6.0 LZW (section 13): MSB-first codes of 9..12 bits, 256 clears
    the table, 257 ends the strip, the code width grows one code early."""
    out = bytearray()
    table = [bytes([i]) for i in range(256)] + [b"", b""]
    width, pos, prev = 9, 0, None
    nbits = len(data) * 8
    while pos + width <= nbits:
        byte, bit = divmod(pos, 8)
        chunk = int.from_bytes(data[byte:byte + 3].ljust(3, b"\0"), "big")
        code = (chunk >> (24 - bit - width)) & ((1 << width) - 1)
        pos += width
        if code == 257:
            break
        if code == 256:
            table = table[:258]
            width, prev = 9, None
            continue
        if prev is None:
            entry = table[code]
        elif code < len(table):
            entry = table[code]
            table.append(prev + entry[:1])
        else:
            entry = prev + prev[:1]
            table.append(entry)
        out += entry
        prev = entry
        if len(table) + 1 >= (1 << width) and width < 12:
            width += 1
    return bytes(out)


def read_tiff(path):
    data = open(path, "rb").read()
    bo = "<" if data[:2] == b"II" else ">"
    (ifd,) = struct.unpack(bo + "I", data[4:8])
    (n,) = struct.unpack(bo + "H", data[ifd:ifd + 2])
    tags = {}
    tsize = {1: 1, 2: 1, 3: 2, 4: 4, 5: 8, 7: 1, 11: 4, 12: 8, 16: 8}
    tfmt = {1: "B", 2: "c", 3: "H", 4: "I", 7: "B", 16: "Q"}
    for i in range(n):
        e = data[ifd + 2 + 12 * i: ifd + 14 + 12 * i]
        tag, typ, cnt = struct.unpack(bo + "HHI", e[:8])
        sz = tsize.get(typ, 1) * cnt
        raw = e[8:12] if sz <= 4 else data[struct.unpack(bo + "I", e[8:12])[0]:][:sz]
        if typ in tfmt:
            vals = struct.unpack(bo + tfmt[typ] * cnt, raw[:sz])
        else:
            vals = raw
        tags[tag] = vals
    W, H = tags[256][0], tags[257][0]
    spp = tags.get(277, (1,))[0]
    bps = tags.get(258, (8,))[0]
    comp = tags.get(259, (1,))[0]
    pred = tags.get(317, (1,))[0]
    offs, cnts = tags[273], tags[279]
    rps = tags.get(278, (H,))[0]
    assert bps == 8, "only 8-bit images are expected"
    rows = []
    for o, c in zip(offs, cnts):
        chunk = data[o:o + c]
        if comp in (8, 32946):
            chunk = zlib.decompress(chunk)
        elif comp == 5:
            chunk = lzw_decode(chunk)
        elif comp != 1:
            raise ValueError("compression %d not supported" % comp)
        rows.append(np.frombuffer(chunk, np.uint8))
    img = np.concatenate(rows)[: W * H * spp].reshape(H, W, spp).copy()
    if pred == 2:
        img = np.cumsum(img.astype(np.uint16), axis=1).astype(np.uint8)
    return img


def read_exr(path):
    """Scanline OpenEXR with ZIP compression (16 lines per block) and HALF
    or FLOAT channels (testshade -od half / float): zlib, then
    undo the byte predictor and the even/odd byte split of the format."""
    d = open(path, "rb").read()
    assert d[:4] == b"\x76\x2f\x31\x01", "not an OpenEXR file"
    i, attrs = 8, {}
    while d[i] != 0:
        n = d.index(b"\0", i)
        name = d[i:n].decode()
        i = n + 1
        n = d.index(b"\0", i)
        i = n + 1
        (sz,) = struct.unpack("<i", d[i:i + 4])
        i += 4
        attrs[name] = d[i:i + sz]
        i += sz
    i += 1
    assert attrs["compression"][0] == 3, "only ZIP compression is read here"
    x0, y0, x1, y1 = struct.unpack("<4i", attrs["dataWindow"])
    W, H = x1 - x0 + 1, y1 - y0 + 1
    chans, ptypes, c = [], [], attrs["channels"]
    j = 0
    while c[j] != 0:
        n = c.index(b"\0", j)
        nm = c[j:n].decode()
        (ptype,) = struct.unpack("<i", c[n + 1:n + 5])
        assert ptype in (1, 2), "only HALF and FLOAT channels are read here"
        assert not chans or ptype == ptypes[0], "one pixel type for every channel"
        chans.append(nm)
        ptypes.append(ptype)
        j = n + 17
    nblocks = (H + 15) // 16
    offsets = struct.unpack("<%dQ" % nblocks, d[i:i + 8 * nblocks])
    img = np.zeros((H, W, len(chans)), np.float32)
    for off in offsets:
        y, size = struct.unpack("<ii", d[off:off + 8])
        raw = np.frombuffer(zlib.decompress(d[off + 8:off + 8 + size]), np.uint8).astype(np.int32)
        t = np.cumsum(np.concatenate([raw[:1], raw[1:] - 128])) & 0xFF
        t = t.astype(np.uint8)
        half = (len(t) + 1) // 2
        inter = np.empty(len(t), np.uint8)
        inter[0::2] = t[:half]
        inter[1::2] = t[half:]
        lines = min(16, H - (y - y0))
        vals = np.frombuffer(inter.tobytes(), np.float16 if ptypes[0] == 1 else np.float32).reshape(lines, len(chans), W)
        img[y - y0:y - y0 + lines] = vals.transpose(0, 2, 1).astype(np.float32)
    return img, chans


EXR_IMAGES = {
    # every reference image of the test: runtest accepts a match with any
    "blackbody": ["testsuite/blackbody/ref/out.exr", "testsuite/blackbody/ref/out.alt.exr",
                  "testsuite/blackbody/ref/out2.exr", "testsuite/blackbody/ref/out3.exr",
                  "testsuite/blackbody/ref/out4.exr", "testsuite/blackbody/ref/out5.exr"],
    # testrender furnace scenes: spheres under a uniform environment
    "furnace_diffuse": ["testsuite/render-furnace-diffuse/ref/out.exr"],
    "furnace_oren_nayar": ["testsuite/render-mx-furnace-oren-nayar/ref/out.exr"],
    "furnace_sheen": ["testsuite/render-mx-furnace-sheen/ref/out.exr"],
    "wavelength_color": ["testsuite/wavelength_color/ref/out.exr"],
}

IMAGES = {
    # fixture name: (reference path, note)
    "noise": "testsuite/noise/ref/out.tif",
    "cellnoise": "testsuite/cellnoise/ref/out.tif",
    "hashnoise": "testsuite/hashnoise/ref/out.tif",
    "hashnoise_alt_batch": "testsuite/hashnoise/ref/out-alt-batch.tif",
    "hashnoise_fma": "testsuite/hashnoise/ref/out_LLVM_JIT_FMA.tif",
    "noise_perlin": "testsuite/noise-perlin/ref/out.tif",
    "noise_cell": "testsuite/noise-cell/ref/out.tif",
    "noise_simplex": "testsuite/noise-simplex/ref/out.tif",
    "noise_gabor": "testsuite/noise-gabor/ref/out.tif",
    "pnoise_gabor": "testsuite/pnoise-gabor/ref/out.tif",
    "noise_gabor2d_filter": "testsuite/noise-gabor2d-filter/ref/out.tif",
    "noise_gabor3d_filter": "testsuite/noise-gabor3d-filter/ref/out.tif",
    "pnoise_perlin": "testsuite/pnoise-perlin/ref/out.tif",
    "pnoise_cell": "testsuite/pnoise-cell/ref/out.tif",
    # testsuite/spline: Cspline, DxCspline, Fspline, DxFspline, NumKnots
    "spline_color": "testsuite/spline/ref/color.tif",
    "spline_dcolor": "testsuite/spline/ref/dcolor.tif",
    "spline_dcolor_alt": "testsuite/spline/ref/dcolor-oiio2.2.tif",
    "spline_float": "testsuite/spline/ref/float.tif",
    "spline_dfloat": "testsuite/spline/ref/dfloat.tif",
    "spline_numknots": "testsuite/spline/ref/numknots.tif",
    "spline_constcolor": "testsuite/spline/ref/constcolor.tif",
    "spline_derivbug_color": "testsuite/spline-derivbug/ref/color.tif",
    "spline_derivbug_dx": "testsuite/spline-derivbug/ref/dx.tif",
    "spline_derivbug_dx_alt": "testsuite/spline-derivbug/ref/dx-oiio2.2.tif",
    "spline_derivbug_dy": "testsuite/spline-derivbug/ref/dy.tif",
    "spline_nonuniform": "testsuite/spline-nonuniformknots/ref/out.tif",
    "splineinverse_ident": "testsuite/splineinverse-ident/ref/out.tif",
}

TEXTS = {
    # fixture file: reference path
    "deformer_out.txt": "testsuite/example-batched-deformer/ref/out.txt",
    "splineinverse_out.txt": "testsuite/splineinverse/ref/out.txt",
    "closure_out.txt": "testsuite/closure/ref/out.txt",
    "closure_zero_out.txt": "testsuite/closure-zero/ref/out.txt",
    "closure_conditional_out.txt": "testsuite/closure-conditional/ref/out.txt",
    "matrix_out.txt": "testsuite/matrix/ref/out.txt",
    "transform_out.txt": "testsuite/transform/ref/out.txt",
    "transformc_out.txt": "testsuite/transformc/ref/out.txt",
    "colorspace_out.txt": "testsuite/colorspace/ref/out.txt",
    "color_out.txt": "testsuite/color/ref/out.txt",
    "raytype_out.txt": "testsuite/raytype/ref/out.txt",
    "isconnected_out.txt": "testsuite/isconnected/ref/out.txt",
    "isconstant_out.txt": "testsuite/isconstant/ref/out.txt",
    "exponential_out.txt": "testsuite/exponential/ref/out.txt",
    "hyperb_out.txt": "testsuite/hyperb/ref/out.txt",
    "gettextureinfo_out.txt": "testsuite/gettextureinfo/ref/out.txt",
    "unknown_instruction_out.txt": "testsuite/unknown-instruction/ref/out.txt",
    "unknown_instruction.oso": "testsuite/unknown-instruction/test.oso",
}


def known_answers():
    src = open(os.path.join(REF, "src/liboslnoise/oslnoise_test.cpp")).read()
    out = {}
    for name in ["results_1d", "results_2d", "results_3d", "results_4d"]:
        for fn in ["test_perlin", "test_cell"]:
            body = src.split("void\n" + fn)[1].split("\n}\n")[0]
            m = re.search(r"static float %s\[[^\]]*\]\s*=\s*\{([^}]*)\}" % name, body)
            if m:
                out[fn + "." + name] = [float(x) for x in m.group(1).replace("\n", " ").split(",") if x.strip()]
        for fn in ["test_perlin", "test_cell"]:
            body = src.split("void\n" + fn)[1].split("\n}\n")[0]
            m = re.search(r"static Vec3 v%s\[[^\]]*\]\s*=\s*\{(.*?)\};" % name, body, re.S)
            if m:
                vecs = re.findall(r"Vec3\(([^)]*)\)", m.group(1))
                out[fn + ".v" + name] = [[float(t) for t in v.split(",")] for v in vecs]
    return out


def main():
    if not os.path.isdir(REF):
        print("reference tree not present; fixtures are already committed")
        return 0
    for name, rel in IMAGES.items():
        img = read_tiff(os.path.join(REF, rel))
        H, W = img.shape[:2]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), img=img[::STEP, ::STEP], full_w=W, full_h=H,
                            step=STEP)
        print(name, img.shape)
    for name, rels in EXR_IMAGES.items():
        imgs = []
        for rel in rels:
            img, chans = read_exr(os.path.join(REF, rel))
            order = [chans.index(c) for c in ("R", "G", "B")]
            imgs.append(img[:, :, order])
        stack = np.stack(imgs)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), imgs=stack, full_w=stack.shape[2],
                            full_h=stack.shape[1])
        print(name, stack.shape)
    for fixture, rel in TEXTS.items():
        open(os.path.join(HERE, fixture), "w").write(open(os.path.join(REF, rel)).read())
    ka = known_answers()
    json.dump(ka, open(os.path.join(HERE, "oslnoise_known.json"), "w"), indent=1)
    print("known answers:", sorted(ka))
    return 0


if __name__ == "__main__":
    if len(sys.argv) > 1:
        REF = sys.argv[1]
    sys.exit(main())
