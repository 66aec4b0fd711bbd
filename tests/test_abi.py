"""The C ABI library loads without a GPU and exports every declared entry point."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import luz_gb300 as L
from luz_gb300 import _abi

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(luz_[a-z0-9_]+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported():
    names = declared_functions()
    assert len(names) > 40
    lib = C.CDLL(str(_abi.LIB_PATH))
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_signature_table_covers_header():
    bound = {n for n, _, _ in _abi.SIGNATURES}
    assert declared_functions() <= bound, declared_functions() - bound


def test_struct_layouts():
    # LuzCommon.h:37-125 (std430): ModelBlock 128 B, the LightBlock fields on the path 64 B.
    assert C.sizeof(_abi.Light) == 64
    assert C.sizeof(_abi.Model) == 128
    assert C.sizeof(_abi.Vertex) == 48
    assert C.sizeof(_abi.Scene) == 480
    assert C.sizeof(_abi.Instance) == 64
    assert _abi.Scene.inverse_proj.offset == 16 + 4 * 64
    assert _abi.Scene.cam_pos.offset == 16 + 6 * 64 + 16


def test_no_device_is_reported_cleanly():
    h = C.c_void_p()
    st = L.lib.luz_ctx_create(0, C.byref(h))
    if st == 0:          # a GPU is present: nothing to check here
        L.lib.luz_ctx_destroy(h)
        return
    assert st == 6       # LUZ_ERR_NO_DEVICE


def test_null_arguments_are_rejected():
    assert L.lib.luz_ctx_create(0, None) == 1
    assert L.lib.luz_ctx_synchronize(None) == 1
    assert L.lib.luz_frame_read(None, None, 0, None, 0) == 1


def test_scene_generators_are_deterministic():
    a = L.HostScene(1, width=32, height=32)
    b = L.HostScene(1, width=32, height=32)
    assert np.array_equal(a.transforms(), b.transforms())
    assert bytes(a.models()) == bytes(b.models())
    assert bytes(a.lights()) == bytes(b.lights())
    c = L.HostScene(1, seed=99, width=32, height=32)
    assert not np.array_equal(a.transforms(), c.transforms())


def test_config1_scene_shape():
    s = L.HostScene(1)
    assert (s.width, s.height) == (512, 512)
    assert s.instance_count == 65
    assert s.triangle_count() == 2 + 64 * 12
    types = [s.lights()[i].type for i in range(s.light_count)]
    assert types.count(L.LIGHT_DIRECTIONAL) == 1 and types.count(L.LIGHT_POINT) == 4
    b = s.block()
    assert b.ao_num_samples == 4 and abs(b.ao_max - 1.0) < 1e-7 and b.shadow_type == L.SHADOW_RAYTRACING
    for v, _ in s.meshes():
        assert np.isfinite(v).all()


def test_config2_scene_shape_small():
    s = L.HostScene(2, width=64, height=36, meshes=3, instances=20, subdivisions=3)
    meshes = s.meshes()
    assert all(len(i) == 3 * 20 * 4 ** 3 for _, i in meshes)
    r = np.linalg.norm(meshes[0][0][:, :3], axis=1)
    assert r.min() > 1.0 - 8 * 0.05 - 1e-5 and r.max() < 1.0 + 8 * 0.05 + 1e-5
    n = np.linalg.norm(meshes[0][0][:, 3:6], axis=1)
    assert np.allclose(n, 1.0, atol=1e-5)
    types = [s.lights()[i].type for i in range(s.light_count)]
    assert types.count(L.LIGHT_POINT) == 32 and types.count(L.LIGHT_SPOT) == 8


def test_icosphere_counts_config2():
    s = L.HostScene(2, width=16, height=16, meshes=1, instances=1)
    (v, i), = s.meshes()
    assert len(i) // 3 == 81920 and len(v) == 40962


def test_blue_noise_substitute():
    t = L.blue_noise(7)
    assert t.shape == (128, 128, 4) and t.dtype == np.uint8
    assert np.array_equal(t, L.blue_noise(7))
    # roughly uniform bytes in R and G
    for c in range(2):
        h = np.bincount(t[..., c].ravel(), minlength=256)
        assert h.max() < 4 * h.mean()


_NULL_SWEEP = r"""
import ctypes as C, json, re, sys
from pathlib import Path
sys.path.insert(0, sys.argv[1])
from luz_gb300 import _abi
root = Path(sys.argv[1])
status = set()
for h in (root / "include").glob("*.h"):
    text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
    status |= set(re.findall(r"^\s*luz_status\s+(luz_[a-z0-9_]+)\s*\(", text, re.M))
lib = C.CDLL(str(_abi.LIB_PATH))
out = {}
for name, restype, argtypes in _abi.SIGNATURES:
    print(name, file=sys.stderr, flush=True)     # the last name printed is the one that crashed
    f = getattr(lib, name)
    f.restype, f.argtypes = restype, argtypes
    args = [0.0 if t in (C.c_float, C.c_double) else
            0 if isinstance(t, type) and issubclass(t, C._SimpleCData) and t not in (C.c_void_p, C.c_char_p)
            else None for t in argtypes]
    r = f(*args)
    if name in status:
        out[name] = r
print(json.dumps(out))
"""


def test_null_and_zero_arguments_never_crash_and_statuses_are_invalid():
    """Every entry point called with NULL pointers and zero sizes returns without
    touching memory; those returning luz_status return LUZ_ERR_INVALID (the check
    comes before any CUDA call, so no GPU is needed)."""
    import json
    import subprocess
    import sys

    r = subprocess.run([sys.executable, "-c", _NULL_SWEEP, str(ROOT)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, "crashed in " + (r.stderr.strip().splitlines() or ["?"])[-1]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert len(res) > 40
    bad = {k: v for k, v in res.items() if v != 1}
    assert not bad, bad


def test_scene_generator_limits_and_host_memory_errors():
    """Parameters past the documented limit return LUZ_ERR_LIMIT, and a scene larger
    than host memory returns LUZ_ERR_OOM through the C ABI (no exception escapes it):
    64 icospheres of 21 M triangles in a process held to 1 GB of address space."""
    import subprocess
    import sys

    with pytest.raises(L.LuzError, match="LUZ_ERR_LIMIT"):
        L.HostScene(2, width=16, height=16, subdivisions=11)
    code = ("import resource, sys; sys.path.insert(0, sys.argv[1]); import luz_gb300 as L\n"
            "resource.setrlimit(resource.RLIMIT_AS, (1 << 30, 1 << 30))\n"
            "try:\n    L.HostScene(2, width=16, height=16, meshes=64, subdivisions=10)\n"
            "except L.LuzError as e:\n    print(e.status)\n")
    r = subprocess.run([sys.executable, "-c", code, str(ROOT)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == "3"   # LUZ_ERR_OOM


def test_headers_are_c_and_link_from_c(tmp_path):
    """include/*.h compile as strict C99, and a C program that takes the address of
    every declared function links against the library and runs (its one call returns
    LUZ_ERR_INVALID for a NULL output, with no GPU)."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    names = sorted(declared_functions())
    src = tmp_path / "abi.c"
    src.write_text('#include "luz.h"\n#include "luz_scene.h"\n#include <stdio.h>\n'
                   "static void (*const table[])(void) = {\n" +
                   "".join(f"    (void (*)(void)){n},\n" for n in names) +
                   "};\nint main(void) {\n"
                   "    printf(\"%d %d\\n\", (int)(sizeof table / sizeof table[0]), (int)luz_ctx_create(0, 0));\n"
                   "    return 0;\n}\n")
    exe = tmp_path / "abi"
    lib = Path(_abi.LIB_PATH)
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-pedantic", "-I", str(ROOT / "include"),
                    str(src), "-o", str(exe), "-L", str(lib.parent), "-l:" + lib.name,
                    "-Wl,-rpath," + str(lib.parent)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == [str(len(names)), "1"]
