#!/usr/bin/env python3
"""Golden fixtures for the scene-file importers and the project format.

Writes small synthetic scene files (our own content: a glTF 2.0 JSON scene with an
embedded PNG texture, the same scene as a GLB, an OBJ + MTL pair) into
tests/golden/ingest/, runs them through the reference renderer's own importers and
project (de)serialiser (oracle/_ref/libluz_ref_ingest.so, built by `make -C oracle
ref` from the reference tree) and stores what the reference produced:

  ref_<file>.json       AssetManager::AddAssetsToScene of the file, packed per MeshNode
                        (world matrix, material, mesh) and LightNode, plus settings
  synth_ref.luz/.luzbin the glTF import saved by AssetManager::SaveProject
  ref_load_synth.json   AssetManager::LoadProject of that pair, packed the same way
  ref_assets.json       digests of the reference repository's own assets (cube.glb,
                        point/spot/directional.obj) through its importer

Run from the repository root where the reference tree exists:
    python tests/golden/make_ingest_golden.py [--reference <reference tree>]
"""
import argparse
import base64
import ctypes as C
import json
import os
import struct
import subprocess
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "ingest")
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle.reference_tree import reference_root  # noqa: E402


def png_bytes(rgba: np.ndarray) -> bytes:
    h, w, _ = rgba.shape
    raw = b"".join(b"\x00" + rgba[y].tobytes() for y in range(h))

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(raw, 9)) + chunk(b"IEND", b""))


def checker(n=16):
    y, x = np.mgrid[0:n, 0:n]
    c = ((x // 4 + y // 4) % 2).astype(np.uint8)
    img = np.zeros((n, n, 4), np.uint8)
    img[..., 0] = 40 + 200 * c
    img[..., 1] = 200 - 150 * c
    img[..., 2] = (x * 16).astype(np.uint8)
    img[..., 3] = 255
    img[0, 0, 3] = 128
    return img


def box_mesh():
    """A unit box: 24 vertices (positions, normals, UVs), 36 indices (u16)."""
    pos, nrm, uv, idx = [], [], [], []
    faces = [((1, 0, 0), (0, 1, 0)), ((-1, 0, 0), (0, 0, 1)), ((0, 1, 0), (0, 0, 1)),
             ((0, -1, 0), (1, 0, 0)), ((0, 0, 1), (1, 0, 0)), ((0, 0, -1), (0, 1, 0))]
    for n, u in faces:
        n, u = np.array(n, np.float32), np.array(u, np.float32)
        v = np.cross(n, u)
        b = len(pos)
        for k, (su, sv) in enumerate([(-1, -1), (1, -1), (1, 1), (-1, 1)]):
            pos.append(0.5 * (n + su * u + sv * v))
            nrm.append(n)
            uv.append(((su + 1) * 0.5, (sv + 1) * 0.5))
        idx += [b, b + 1, b + 2, b, b + 2, b + 3]
    return (np.array(pos, np.float32), np.array(nrm, np.float32), np.array(uv, np.float32),
            np.array(idx, np.uint16))


def tri_fan(n=7):
    """A flat n-gon fan with per-vertex tangents given (u32 indices)."""
    ang = np.linspace(0, 2 * np.pi, n, endpoint=False)
    pos = np.concatenate([[[0, 0, 0]], np.stack([np.cos(ang), np.zeros(n), np.sin(ang)], 1)]).astype(np.float32)
    nrm = np.tile(np.array([[0, 1, 0]], np.float32), (n + 1, 1))
    tan = np.tile(np.array([[1, 0, 0, 1]], np.float32), (n + 1, 1))
    uv = (pos[:, [0, 2]] * 0.5 + 0.5).astype(np.float32)
    idx = np.array([[0, 1 + k, 1 + (k + 1) % n] for k in range(n)], np.uint32).ravel()
    return pos, nrm, tan, uv, idx


def gltf_scene():
    """glTF JSON dict + one binary buffer."""
    bp, bn, bu, bi = box_mesh()
    fp, fn, ft, fu, fi = tri_fan()
    png = png_bytes(checker())
    blobs, views, accs = [], [], []

    def add(arr, target=None):
        off = sum(len(b) for b in blobs)
        data = arr.tobytes()
        pad = (-len(data)) % 4
        blobs.append(data + b"\0" * pad)
        v = {"buffer": 0, "byteOffset": off, "byteLength": len(data)}
        if target:
            v["target"] = target
        views.append(v)
        return len(views) - 1

    def acc(arr, ctype, typ):
        vi = add(arr)
        a = {"bufferView": vi, "componentType": ctype, "count": int(arr.shape[0]), "type": typ}
        if typ == "VEC3" and ctype == 5126:
            a["min"] = arr.min(0).tolist()
            a["max"] = arr.max(0).tolist()
        accs.append(a)
        return len(accs) - 1

    box = {"POSITION": acc(bp, 5126, "VEC3"), "NORMAL": acc(bn, 5126, "VEC3"), "TEXCOORD_0": acc(bu, 5126, "VEC2")}
    box_i = acc(bi, 5123, "SCALAR")
    fan = {"POSITION": acc(fp, 5126, "VEC3"), "NORMAL": acc(fn, 5126, "VEC3"), "TANGENT": acc(ft, 5126, "VEC4"),
           "TEXCOORD_0": acc(fu, 5126, "VEC2")}
    fan_i = acc(fi, 5125, "SCALAR")
    img_view = add(np.frombuffer(png, np.uint8))
    q = np.array([0.2, -0.3, 0.1, 0.927], np.float64)
    q /= np.linalg.norm(q)
    m = np.eye(4)
    m[:3, 3] = [1.5, 0.25, -2.0]
    m[:3, :3] = np.diag([2.0, 0.5, 1.25])
    gj = {
        "asset": {"version": "2.0", "generator": "luz_gb300 golden fixtures"},
        "scene": 0,
        "scenes": [{"name": "Synth", "nodes": [0, 3]}],
        "nodes": [
            {"name": "Root", "translation": [0.5, 1.0, -0.25], "rotation": q.tolist(), "scale": [1.5, 1.5, 1.5],
             "children": [1, 2]},
            {"name": "Box", "mesh": 0, "translation": [2.0, 0.0, 0.0], "rotation": [0.0, 0.38268343, 0.0, 0.92387953]},
            {"name": "Fan", "mesh": 1, "matrix": m.T.ravel().tolist()},
            {"name": "Lamp", "translation": [0.0, 5.0, 1.0], "rotation": [-0.70710677, 0.0, 0.0, 0.70710677],
             "extensions": {"KHR_lights_punctual": {"light": 0}}},
        ],
        "meshes": [{"name": "Box", "primitives": [{"attributes": box, "indices": box_i, "material": 0}]},
                   {"name": "Fan", "primitives": [{"attributes": fan, "indices": fan_i, "material": 1}]}],
        "materials": [
            {"name": "Checker", "pbrMetallicRoughness": {"baseColorTexture": {"index": 0}, "metallicFactor": 0.25,
                                                         "roughnessFactor": 0.75},
             "emissiveFactor": [0.1, 0.0, 0.05]},
            {"name": "Plain", "pbrMetallicRoughness": {"baseColorFactor": [0.8, 0.3, 0.2, 1.0]}},
        ],
        "textures": [{"name": "checker", "source": 0}],
        "images": [{"bufferView": img_view, "mimeType": "image/png"}],
        "extensionsUsed": ["KHR_lights_punctual"],
        "extensions": {"KHR_lights_punctual": {"lights": [{"type": "point", "intensity": 3.0}]}},
        "bufferViews": views,
        "accessors": accs,
    }
    binary = b"".join(blobs)
    gj["buffers"] = [{"byteLength": len(binary)}]
    return gj, binary


def write_gltf(gj, binary, path):
    g = json.loads(json.dumps(gj))
    g["buffers"][0]["uri"] = "data:application/octet-stream;base64," + base64.b64encode(binary).decode()
    with open(path, "w") as f:
        json.dump(g, f, indent=1)


def write_glb(gj, binary, path):
    js = json.dumps(gj).encode()
    js += b" " * ((-len(js)) % 4)
    binary += b"\0" * ((-len(binary)) % 4)
    body = struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(binary), 0x004E4942) + binary
    with open(path, "wb") as f:
        f.write(struct.pack("<III", 0x46546C67, 2, 12 + len(body)) + body)


def write_obj(path_obj, path_mtl):
    with open(path_mtl, "w") as f:
        f.write("# synthetic material library\n"
                "newmtl red\nKd 0.9 0.1 0.1\nKs 0 0 0\nKe 0.0 0.0 0.0\nPm 0.5\nPr 0.3\n\n"
                "newmtl shiny\nKd 0.2 0.2 0.9\nKs 0.6 0.6 0.9\nPm 0.0\n")
    lines = ["# synthetic OBJ: quads, triangles, negative indices, all index forms",
             f"mtllib {os.path.basename(path_mtl)}", "o Slab"]
    for y in (0.0, 1.0):
        for z in (0.0, 1.0, 2.0):
            for x in (0.0, 1.0, 2.0):
                lines.append(f"v {x:.6f} {y:.6f} {z:.6f}")
    for u, v in ((0, 0), (1, 0), (1, 1), (0, 1), (0.5, 0.5)):
        lines.append(f"vt {u:.6f} {v:.6f}")
    for n in ((0, -1, 0), (0, 1, 0), (0, 0, 1)):
        lines.append("vn %.6f %.6f %.6f" % n)
    lines.append("usemtl red")
    lines.append("f 1/1/1 2/2/1 5/3/1 4/4/1")          # quad with v/vt/vn
    lines.append("f 2//1 3//1 6//1 5//1")              # quad with v//vn
    lines.append("f 10/1 11/2 14/3")                   # triangle with v/vt
    lines.append("f 11 12 15 14")                      # quad, positions only
    lines.append("f -8/-5/-2 -7/-4/-2 -4/-3/-2")       # negative (relative) indices
    lines.append("o Cap")
    lines.append("usemtl shiny")
    lines.append("f 4/1/3 5/2/3 8/3/3 7/4/3")
    lines.append("f 5/2/3 6/5/3 9/3/3 8/4/3")
    with open(path_obj, "w") as f:
        f.write("\n".join(lines) + "\n")


def digest_assets(lib, ref_root):
    """The reference's own assets through its importer: per mesh the counts, CRCs of
    the position/normal/texcoord columns, of the tangents, of the indices, and the
    CRC of the sorted set of unique vertices."""
    out = {}
    for name in ("cube.glb", "point.obj", "spot.obj", "directional.obj"):
        src = os.path.join(ref_root, "assets", name)
        if not os.path.exists(src):
            continue
        tmp = os.path.join(OUT, "_tmp.json")
        lib.ref_import_dump(src.encode(), tmp.encode())
        d = json.load(open(tmp))
        os.unlink(tmp)
        meshes = []
        for m in d["meshes"]:
            v = np.array(m["vertices"], np.float32).reshape(-1, 12)
            i = np.array(m["indices"], np.uint32)
            meshes.append(mesh_digest(v, i))
        out[name] = {"instances": d["instances"], "textures": d["textures"], "lights": d["lights"],
                     "meshes": meshes}
    return out


def mesh_digest(v: np.ndarray, i: np.ndarray) -> dict:
    cols = np.ascontiguousarray(v[:, [0, 1, 2, 3, 4, 5, 10, 11]])
    uniq = sorted(set(map(bytes, np.ascontiguousarray(v).view(np.uint32))))
    p = v[:, :3].astype(np.float64)[i.reshape(-1, 3)]
    area = 0.5 * np.linalg.norm(np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), axis=1).sum()
    return {"vertex_count": int(v.shape[0]), "index_count": int(i.size),
            "crc_pnt": zlib.crc32(cols.tobytes()), "crc_tangent": zlib.crc32(np.ascontiguousarray(v[:, 6:10]).tobytes()),
            "tangent_absmax": float(np.abs(v[:, 6:10]).max()) if v.size else 0.0,
            "crc_indices": zlib.crc32(i.astype(np.uint32).tobytes()),
            "crc_unique_vertices": zlib.crc32(b"".join(uniq)), "area": float(area)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=reference_root())
    args = ap.parse_args()
    if not args.reference:
        sys.exit("the reference tree was not found: set LUZ_REF_ROOT or pass --reference")
    os.makedirs(OUT, exist_ok=True)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"LUZ_REF_ROOT={args.reference}"],
                   check=True)
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libluz_ref_ingest.so"), mode=C.RTLD_GLOBAL)
    gj, binary = gltf_scene()
    files = {"synth.gltf": lambda p: write_gltf(gj, binary, p), "synth.glb": lambda p: write_glb(gj, binary, p),
             "synth.obj": lambda p: write_obj(p, os.path.join(OUT, "synth.mtl"))}
    for name, make in files.items():
        path = os.path.join(OUT, name)
        make(path)
        lib.ref_import_dump(path.encode(), os.path.join(OUT, f"ref_{name}.json").encode())
    luz, luzbin = os.path.join(OUT, "synth_ref.luz"), os.path.join(OUT, "synth_ref.luzbin")
    lib.ref_save_import(os.path.join(OUT, "synth.gltf").encode(), luz.encode(), luzbin.encode())
    lib.ref_load_dump(luz.encode(), luzbin.encode(), os.path.join(OUT, "ref_load_synth.json").encode())
    with open(os.path.join(OUT, "ref_assets.json"), "w") as f:
        json.dump(digest_assets(lib, args.reference), f, indent=0)
    print("wrote", sorted(os.listdir(OUT)))


if __name__ == "__main__":
    sys.exit(main())
