"""Scene files: the .luz/.luzbin project format, glTF 2.0 and OBJ importers.

Golden fixtures (tests/golden/ingest/, made by make_ingest_golden.py) hold what the
reference renderer's own importers and project loader produced for synthetic scene
files and for the reference repository's assets. Bit-exact: meshes (positions,
normals, texcoords, indices), world matrices, materials, textures (CRC of the
decoded RGBA8), tangents read from a file. Tangents that the glTF importer computes
are checked for their properties instead (unit length, orthogonal to the normal,
handedness +-1): the reference accumulates them in uninitialised memory
(`new glm::vec3[]`, source/Resources/AssetIO.cpp:327), so its own values vary from
run to run (stray denormals, sometimes NaN or wrong signs).
"""
import ctypes as C
import json
import os
import struct
import zlib

import numpy as np
import pytest

import luz_gb300 as L
from oracle.reference_tree import reference_root

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "ingest")
REF_ROOT = reference_root()
REF_LIB = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libluz_ref_ingest.so")


def gold(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def bits(a):
    return np.ascontiguousarray(np.asarray(a, np.float32)).view(np.uint32)


def check_computed_tangents(v):
    t, n, w = v[:, 6:9].astype(np.float64), v[:, 3:6].astype(np.float64), v[:, 9]
    assert np.allclose(np.linalg.norm(t, axis=1), 1.0, atol=1e-6)
    assert np.allclose(np.sum(t * n, axis=1), 0.0, atol=1e-6)
    assert np.all(np.abs(w) == 1.0)


def check_mesh(ref_v, ref_i, ov, oi, computed_tangents=False):
    rv = np.array(ref_v, np.float32).reshape(-1, 12)
    assert rv.shape == ov.shape
    assert np.array_equal(np.asarray(ref_i, np.uint32), oi)
    cols = [0, 1, 2, 3, 4, 5, 10, 11]
    assert np.array_equal(bits(rv[:, cols]), bits(ov[:, cols]))
    if computed_tangents:
        check_computed_tangents(ov)
    else:
        rt, ot = rv[:, 6:10], ov[:, 6:10]
        both_nan = np.isnan(rt) & np.isnan(ot)   # the dump keeps no NaN payload
        assert np.array_equal(bits(np.where(both_nan, 0, rt)), bits(np.where(both_nan, 0, ot)))


def check_scene(ref, s: L.HostScene, computed=()):
    models, meshes, im = s.models(), s.meshes(), s.instance_mesh()
    assert len(ref["instances"]) == s.instance_count
    texcrc = [zlib.crc32(t.tobytes()) for t in s.textures()]
    for k, inst in enumerate(ref["instances"]):
        m = models[k]
        assert np.array_equal(bits(inst["world"]), bits(list(m.model_mat)))
        assert im[k] == inst["mesh"]
        mat = inst.get("material")
        if mat:
            assert np.array_equal(bits(mat["color"]), bits(list(m.color)))
            assert np.array_equal(bits(mat["emission"]), bits(list(m.emission)))
            assert np.float32(mat["metallic"]) == np.float32(m.metallic)
            assert np.float32(mat["roughness"]) == np.float32(m.roughness)
            for key, ours in (("colorMap", m.color_map), ("normalMap", m.normal_map),
                              ("metallicRoughnessMap", m.metallic_roughness_map), ("emissionMap", m.emission_map)):
                if mat[key] < 0:
                    assert ours == -1
                else:
                    assert texcrc[ours] == ref["textures"][mat[key]]["crc32"]
        else:
            assert list(m.color) == [1.0, 1.0, 1.0, 1.0] and m.color_map == -1
    for k, rm in enumerate(ref["meshes"]):
        check_mesh(rm["vertices"], rm["indices"], *meshes[k], computed_tangents=k in computed)
    lights = s.lights()
    assert len(ref["lights"]) == s.light_count
    for k, rl in enumerate(ref["lights"]):
        ol = lights[k]
        assert np.array_equal(bits(rl["position"]), bits(list(ol.position)))
        assert np.allclose(rl["direction"], list(ol.direction), atol=1e-7)
        assert np.float32(rl["intensity"]) == np.float32(ol.intensity) and rl["type"] == ol.type
        assert np.float32(rl["innerAngle"]) == np.float32(ol.inner_angle)
    b = s.block()
    sc = ref["scene"]
    assert np.float32(sc["ambientLight"]) == np.float32(b.ambient_light_intensity)
    assert sc["aoSamples"] == b.ao_num_samples and sc["shadowType"] == b.shadow_type
    assert np.float32(sc["aoMin"]) == np.float32(b.ao_min) and np.float32(sc["aoMax"]) == np.float32(b.ao_max)
    assert all(lights[k].num_shadow_samples == (sc["lightSamples"] if sc["shadowType"] == 1 else 0)
               for k in range(s.light_count))


@pytest.mark.parametrize("name", ["synth.gltf", "synth.glb", "synth.obj"])
def test_import_matches_reference_importer(name):
    s = L.HostScene.import_file(os.path.join(GOLD, name), 320, 240)
    # the box of the glTF scene has no TANGENT attribute
    check_scene(gold(f"ref_{name}.json"), s, computed=(0,) if name != "synth.obj" else ())


def test_gltf_and_glb_agree():
    a = L.HostScene.import_file(os.path.join(GOLD, "synth.gltf"), 64, 64)
    b = L.HostScene.import_file(os.path.join(GOLD, "synth.glb"), 64, 64)
    for (va, ia), (vb, ib) in zip(a.meshes(), b.meshes()):
        assert np.array_equal(bits(va), bits(vb)) and np.array_equal(ia, ib)
    assert [t.tobytes() for t in a.textures()] == [t.tobytes() for t in b.textures()]


def test_load_project_written_by_reference():
    """A .luz/.luzbin pair written by the reference's SaveProject, read back here,
    equals what the reference's LoadProject reads from it."""
    s = L.HostScene.load_project(os.path.join(GOLD, "synth_ref.luz"), os.path.join(GOLD, "synth_ref.luzbin"),
                                 320, 240)
    ref = gold("ref_load_synth.json")
    check_scene(ref, s)   # tangents come from the file here: bit for bit too


def test_project_round_trip(tmp_path):
    """Generated scene -> .luz/.luzbin -> loaded scene: meshes, ModelBlocks and lights
    bit for bit; the camera reproduces the same view."""
    s = L.HostScene(1, width=96, height=64)
    luz, luzbin = tmp_path / "g.luz", tmp_path / "g.luzbin"
    s.save_project(luz, luzbin)
    t = L.HostScene.load_project(luz, luzbin, 96, 64)
    for (va, ia), (vb, ib) in zip(s.meshes(), t.meshes()):
        assert np.array_equal(bits(va), bits(vb)) and np.array_equal(ia, ib)
    assert s.instance_count == t.instance_count
    ma, mb = s.models(), t.models()
    for k in range(s.instance_count):
        assert bytes(ma[k]) == bytes(mb[k])
    la, lb = s.lights(), t.lights()
    for k in range(s.light_count):
        assert bytes(la[k]) == bytes(lb[k])
    ba, bb = s.block(), t.block()
    assert np.allclose(list(ba.view_proj), list(bb.view_proj), rtol=1e-4, atol=1e-4)
    assert np.allclose(list(ba.cam_pos), list(bb.cam_pos), rtol=1e-5, atol=1e-4)
    assert ba.ao_num_samples == bb.ao_num_samples and ba.ao_max == bb.ao_max


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference importer not built (no reference tree)")
def test_reference_loads_our_project(tmp_path):
    """The reference's LoadProject reads a project this library wrote: same meshes,
    materials and lights; world matrices within 1e-5 (it rebuilds them from the
    position / Euler rotation / scale fields)."""
    s = L.HostScene(1, width=96, height=64)
    luz, luzbin, out = tmp_path / "g.luz", tmp_path / "g.luzbin", tmp_path / "dump.json"
    s.save_project(luz, luzbin)
    lib = C.CDLL(REF_LIB, mode=C.RTLD_GLOBAL)
    lib.ref_load_dump(str(luz).encode(), str(luzbin).encode(), str(out).encode())
    ref = json.load(open(out))
    models, meshes, im = s.models(), s.meshes(), s.instance_mesh()
    assert len(ref["instances"]) == s.instance_count
    for k, inst in enumerate(ref["instances"]):
        assert np.allclose(inst["world"], list(models[k].model_mat), atol=1e-5)
        assert np.array_equal(bits(inst["material"]["color"]), bits(list(models[k].color)))
        rm = ref["meshes"][inst["mesh"]]
        ov, oi = meshes[im[k]]
        assert np.array_equal(bits(np.array(rm["vertices"]).reshape(-1, 12)), bits(ov))
        assert np.array_equal(np.asarray(rm["indices"], np.uint32), oi)
    for k, rl in enumerate(ref["lights"]):
        ol = s.lights()[k]
        assert np.array_equal(bits(rl["position"]), bits(list(ol.position)))
        d = np.asarray(list(ol.direction), np.float64)
        assert np.allclose(np.asarray(rl["direction"]) / np.linalg.norm(rl["direction"]), d / np.linalg.norm(d),
                           atol=1e-5)


def _digest(v, i):
    cols = np.ascontiguousarray(v[:, [0, 1, 2, 3, 4, 5, 10, 11]])
    uniq = sorted(set(map(bytes, np.ascontiguousarray(v).view(np.uint32))))
    p = v[:, :3].astype(np.float64)[i.reshape(-1, 3)]
    area = 0.5 * np.linalg.norm(np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), axis=1).sum()
    return cols, uniq, area


@pytest.mark.parametrize("name", ["cube.glb", "point.obj", "spot.obj", "directional.obj"])
def test_reference_assets(name):
    """The reference repository's own assets: digests of what its importer made."""
    path = os.path.join(REF_ROOT, "assets", name) if REF_ROOT else None
    if path is None or not os.path.exists(path):
        pytest.skip("reference assets not present")
    g = gold("ref_assets.json")[name]
    s = L.HostScene.import_file(path, 64, 64)
    assert [zlib.crc32(t.tobytes()) for t in s.textures()] == [t["crc32"] for t in g["textures"]]
    for gm, (v, i) in zip(g["meshes"], s.meshes()):
        assert v.shape[0] == gm["vertex_count"] and i.size == gm["index_count"]
        cols, uniq, area = _digest(v, i)
        if name == "directional.obj":
            # one 32-gon: ear clipping here, tinyobjloader's own clipping there — the
            # same vertices and the same covered area, other diagonals
            assert abs(area - gm["area"]) <= 1e-9 * gm["area"]
            assert len(set(map(bytes, bits(v)))) == len(uniq)
        else:
            assert zlib.crc32(cols.tobytes()) == gm["crc_pnt"]
            assert zlib.crc32(i.astype(np.uint32).tobytes()) == gm["crc_indices"]
        if name == "cube.glb":
            check_computed_tangents(v)
        else:
            assert not v[:, 6:10].any()   # OBJ meshes carry no tangents
    for gi, m in zip(g["instances"], s.models()):
        assert np.array_equal(bits(gi["world"]), bits(list(m.model_mat)))


# ---------------------------------------------------------------- PNG decoding
def _chunk(t, d):
    return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)


def _png(w, h, depth, ctype, rows, plte=None, trns=None, interlace=0):
    out = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, interlace))
    if plte is not None:
        out += _chunk(b"PLTE", plte)
    if trns is not None:
        out += _chunk(b"tRNS", trns)
    raw = b"".join(rows)
    half = len(raw) // 2
    comp = zlib.compress(raw, 9)
    return out + _chunk(b"IDAT", comp[: len(comp) // 2]) + _chunk(b"IDAT", comp[len(comp) // 2:]) + _chunk(b"IEND", b"")


def _pack_row(vals, depth):
    if depth >= 8:
        return bytes(np.asarray(vals, ">u2" if depth == 16 else np.uint8).tobytes())
    out, acc, n = bytearray(), 0, 0
    for v in vals:
        acc = (acc << depth) | int(v)
        n += depth
        if n == 8:
            out.append(acc)
            acc, n = 0, 0
    if n:
        out.append(acc << (8 - n))
    return bytes(out)


def _filtered(rows, bpp, kinds):
    """Applies the PNG filters (one kind per row) to raw rows -> filtered bytes."""
    out, prev = [], bytes(len(rows[0]))
    for r, f in zip(rows, kinds):
        cur = bytearray()
        for x in range(len(r)):
            a = r[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            if f == 0:
                pr = 0
            elif f == 1:
                pr = a
            elif f == 2:
                pr = b
            elif f == 3:
                pr = (a + b) >> 1
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pr = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
            cur.append((r[x] - pr) & 0xFF)
        out.append(bytes([f]) + bytes(cur))
        prev = r
    return out


def _import_png(tmp_path, png: bytes) -> np.ndarray:
    """Decodes through the glTF importer: a one-triangle scene whose material's base
    colour texture is `png`."""
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    idx = np.array([0, 1, 2], np.uint32)
    blob = pos.tobytes() + idx.tobytes() + png
    g = {"asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": [0]}], "nodes": [{"mesh": 0}],
         "meshes": [{"primitives": [{"attributes": {"POSITION": 0}, "indices": 1, "material": 0}]}],
         "materials": [{"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}}}],
         "textures": [{"source": 0}], "images": [{"bufferView": 2, "mimeType": "image/png"}],
         "buffers": [{"byteLength": len(blob), "uri": "data:application/octet-stream;base64," +
                      __import__("base64").b64encode(blob).decode()}],
         "bufferViews": [{"buffer": 0, "byteOffset": 0, "byteLength": 36},
                         {"buffer": 0, "byteOffset": 36, "byteLength": 12},
                         {"buffer": 0, "byteOffset": 48, "byteLength": len(png)}],
         "accessors": [{"bufferView": 0, "componentType": 5126, "count": 3, "type": "VEC3"},
                       {"bufferView": 1, "componentType": 5125, "count": 3, "type": "SCALAR"}]}
    p = tmp_path / "png_probe.gltf"
    p.write_text(json.dumps(g))
    return L.HostScene.import_file(p, 8, 8).textures()[0]


@pytest.mark.parametrize("depth,ctype", [(1, 0), (2, 0), (4, 0), (8, 0), (16, 0), (8, 2), (16, 2), (8, 4),
                                         (16, 4), (8, 6), (16, 6), (1, 3), (4, 3), (8, 3)])
def test_png_formats(tmp_path, depth, ctype):
    rng = np.random.default_rng(depth * 10 + ctype)
    w, h = 13, 7
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    maxv = (1 << depth) - 1
    if ctype == 3:
        maxv = min(maxv, 9)
    samples = rng.integers(0, maxv + 1, size=(h, w, ch))
    plte = trns = None
    if ctype == 3:
        pal = rng.integers(0, 256, size=(maxv + 1, 3), dtype=np.uint8)
        plte = pal.tobytes()
        tr = rng.integers(0, 256, size=maxv // 2 + 1, dtype=np.uint8)
        trns = tr.tobytes()
    rows = [_pack_row(samples[y].ravel(), depth) for y in range(h)]
    bpp = max(1, ch * depth // 8)
    png = _png(w, h, depth, ctype, _filtered(rows, bpp, [y % 5 for y in range(h)]), plte, trns)
    got = _import_png(tmp_path, png)
    want = np.zeros((h, w, 4), np.uint8)
    hi = (samples >> 8) if depth == 16 else samples
    scale = {1: 255, 2: 0x55, 4: 0x11}.get(depth, 1)
    if ctype == 0:
        want[..., :3] = (hi[..., :1] * (scale if depth < 8 else 1)).astype(np.uint8)
        want[..., 3] = 255
    elif ctype == 2:
        want[..., :3] = hi
        want[..., 3] = 255
    elif ctype == 4:
        want[..., :3] = hi[..., :1]
        want[..., 3] = hi[..., 1]
    elif ctype == 6:
        want[...] = hi
    else:
        idx = samples[..., 0]
        want[..., :3] = pal[idx]
        full_tr = np.full(maxv + 1, 255, np.uint8)
        full_tr[: len(tr)] = tr
        want[..., 3] = full_tr[idx]
    assert np.array_equal(got, want)


def test_png_adam7_and_stored_blocks(tmp_path):
    rng = np.random.default_rng(5)
    w, h = 11, 9
    img = rng.integers(0, 256, size=(h, w, 4), dtype=np.uint8)
    passes = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
    raw = b""
    for x0, y0, dx, dy in passes:
        sub = img[y0::dy, x0::dx]
        if sub.size == 0:
            continue
        rows = [sub[y].tobytes() for y in range(sub.shape[0])]
        raw += b"".join(_filtered(rows, 4, [(y + x0) % 5 for y in range(len(rows))]))
    # zlib level 0: stored blocks only
    png = (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 1)) +
           _chunk(b"IDAT", zlib.compress(raw, 0)) + _chunk(b"IEND", b""))
    assert np.array_equal(_import_png(tmp_path, png), img)


def test_png_header_larger_than_its_data_is_rejected_before_allocating(tmp_path):
    """A 65536 x 65536 RGBA header over 64 bytes of image data: every scanline the
    header implies must be decoded before the 16 GiB image is allocated, so the file
    is rejected at once."""
    png = (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", 65536, 65536, 8, 6, 0, 0, 0)) +
           _chunk(b"IDAT", zlib.compress(bytes(64))) + _chunk(b"IEND", b""))
    with pytest.raises(L.LuzError, match="short image data"):
        _import_png(tmp_path, png)


@pytest.mark.parametrize("interlace", [0, 1])
def test_png_data_beyond_the_image_is_not_decoded(tmp_path, interlace):
    """The image's scanlines followed by 64 MB of zeros in one zlib stream (64 KB
    compressed): decoding stops at the size the header implies and the image comes
    from its own scanlines."""
    img = np.arange(2 * 3 * 4, dtype=np.uint8).reshape(2, 3, 4)
    if interlace:   # 3x2 under Adam7: passes 1, 2 (none), 3 (none), 4 (x = 2), 5 (none), 6 (x = 1), 7 (row 1)
        raw = (b"\x00" + img[0, 0].tobytes() + b"\x00" + img[0, 2].tobytes() + b"\x00" + img[0, 1].tobytes() +
               b"\x00" + img[1].tobytes())
    else:
        raw = b"".join(b"\x00" + img[y].tobytes() for y in range(2))
    png = (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", 3, 2, 8, 6, 0, 0, interlace)) +
           _chunk(b"IDAT", zlib.compress(raw + bytes(64 << 20), 9)) + _chunk(b"IEND", b""))
    assert np.array_equal(_import_png(tmp_path, png), img)


def _triangle_gltf(tmp_path, view0=None, acc0=None):
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    blob = pos.tobytes() + np.array([0, 1, 2], np.uint32).tobytes()
    g = {"asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": [0]}], "nodes": [{"mesh": 0}],
         "meshes": [{"primitives": [{"attributes": {"POSITION": 0}, "indices": 1}]}],
         "buffers": [{"byteLength": len(blob), "uri": "data:application/octet-stream;base64," +
                      __import__("base64").b64encode(blob).decode()}],
         "bufferViews": [dict({"buffer": 0, "byteOffset": 0, "byteLength": 36}, **(view0 or {})),
                         {"buffer": 0, "byteOffset": 36, "byteLength": 12}],
         "accessors": [dict({"bufferView": 0, "componentType": 5126, "count": 3, "type": "VEC3"}, **(acc0 or {})),
                       {"bufferView": 1, "componentType": 5125, "count": 3, "type": "SCALAR"}]}
    p = tmp_path / "tri.gltf"
    p.write_text(json.dumps(g))
    return p


@pytest.mark.parametrize("view0,acc0,match", [
    ({"byteOffset": 2 ** 64 - 1, "byteLength": 2}, None, "bufferView outside"),     # offset + length wraps
    (None, {"count": 2 ** 62 + 1}, "accessor outside"),                             # (count - 1) * 12 wraps
    (None, {"byteOffset": 2 ** 64 - 8}, "accessor outside"),
    ({"byteStride": 4}, None, "byteStride smaller"),
    (None, {"byteOffset": -4}, "non-negative"),
    (None, {"count": 1e300}, "non-negative"),
])
def test_gltf_ranges_that_overflow_are_rejected(tmp_path, view0, acc0, match):
    """Offsets, lengths and counts near 2^64 (whose sums or products wrap), negative or
    out-of-range numbers and strides shorter than an element: each is an error, and
    nothing outside the file's buffers is read."""
    assert L.HostScene.import_file(_triangle_gltf(tmp_path), 8, 8).instance_count == 1
    with pytest.raises(L.LuzError, match=match):
        L.HostScene.import_file(_triangle_gltf(tmp_path, view0, acc0), 8, 8)


@pytest.mark.parametrize("face,match", [
    ("f 1 2 4294967297", "missing vertex"),          # would wrap to index 0 in 32 bits
    ("f 1 2 -4", "missing vertex"),
    ("f 1 2 99999999999999999999999", "missing vertex"),
    ("f 1/1 2/1 3/4294967298", "missing texcoord"),
    ("f 1/1 2/1 3/-2", "missing texcoord"),
    ("f 1//1 2//1 3//-3", "missing normal"),
])
def test_obj_indices_outside_what_was_read_are_rejected(tmp_path, face, match):
    """OBJ indices are 1-based or count back from the last element read; any index
    outside that range is an error (none wraps around to a valid element)."""
    good = "v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvn 0 0 1\n"
    (tmp_path / "ok.obj").write_text(good + "f 1/1/1 2/1/1 -1/-1/-1\n")
    assert L.HostScene.import_file(tmp_path / "ok.obj", 8, 8).instance_count == 1
    (tmp_path / "bad.obj").write_text(good + face + "\n")
    with pytest.raises(L.LuzError, match=match):
        L.HostScene.import_file(tmp_path / "bad.obj", 8, 8)


@pytest.mark.parametrize("chain", [512, 513, 100000])
def test_gltf_node_chain_depth(tmp_path, chain):
    """glTF nodes link by index, so a hierarchy can be deeper than its JSON. A chain of
    nodes ending in the mesh's node, whose primitive becomes a MeshNode one level
    further down, loads while that MeshNode is at most 512 levels below the root
    node, and longer chains are rejected without exhausting the stack."""
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    blob = pos.tobytes() + np.array([0, 1, 2], np.uint32).tobytes()
    g = {"asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": [0]}],
         "nodes": [{"children": [i + 1]} for i in range(chain - 1)] + [{"mesh": 0}],
         "meshes": [{"primitives": [{"attributes": {"POSITION": 0}, "indices": 1}]}],
         "buffers": [{"byteLength": len(blob), "uri": "data:application/octet-stream;base64," +
                      __import__("base64").b64encode(blob).decode()}],
         "bufferViews": [{"buffer": 0, "byteOffset": 0, "byteLength": 36},
                         {"buffer": 0, "byteOffset": 36, "byteLength": 12}],
         "accessors": [{"bufferView": 0, "componentType": 5126, "count": 3, "type": "VEC3"},
                       {"bufferView": 1, "componentType": 5125, "count": 3, "type": "SCALAR"}]}
    p = tmp_path / "chain.gltf"
    p.write_text(json.dumps(g))
    if chain <= 512:
        assert L.HostScene.import_file(p, 8, 8).instance_count == 1
    else:
        with pytest.raises(L.LuzError, match="too deep"):
            L.HostScene.import_file(p, 8, 8)


def test_errors_are_reported(tmp_path):
    bad = tmp_path / "bad.gltf"
    bad.write_text("{ not json")
    with pytest.raises(L.LuzError, match="JSON"):
        L.HostScene.import_file(bad)
    with pytest.raises(L.LuzError, match="cannot open"):
        L.HostScene.import_file(tmp_path / "missing.obj")
    with pytest.raises(L.LuzError):
        L.HostScene.import_file(tmp_path / "scene.fbx")
    trunc = tmp_path / "t.png.gltf"
    png = _png(4, 4, 8, 6, [b"\x00" + bytes(16)] * 4)[:-30]
    with pytest.raises(L.LuzError, match="PNG"):
        _import_png(tmp_path, png)
    luz = tmp_path / "x.luz"
    luz.write_text(json.dumps({"assets": [{"type": 2, "uuid": 5, "name": "m",
                                           "vertices": {"offset": 0, "size": 4800}, "indices": {"offset": 0, "size": 0}}],
                               "scenes": {}, "initialScene": 0}))
    (tmp_path / "x.luzbin").write_bytes(b"\0" * 100)
    with pytest.raises(L.LuzError, match="outside"):
        L.HostScene.load_project(luz, tmp_path / "x.luzbin")
