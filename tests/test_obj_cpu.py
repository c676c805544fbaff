"""OBJ / MTL reading of the C++ host adapter (crg::host::load_model, the
counterpart of cr::asset_loader::load_model, src/util/asset_loader.cpp:182-303)
against a small independent restatement of the same rules, on a file that uses
every record form the loader handles."""
import os
import subprocess

import numpy as np
import pytest

EXE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "crender_gb300", "_build",
                   "crg_host_selftest")

MTL = """# two materials
newmtl red
Kd 0.8 0.1 0.1
newmtl grey
Kd 0.5
map_Kd -bm 1.0 textures/grey.png
"""

OBJ = """# test model
mtllib test.mtl
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 2 0 0.5
v 3 0 0.5
v 3 3 0.5
v 2 1 0.5
v 0 0 2
v 1 0 2
v 1.5 0.7 2
v 1 1.4 2
v 0 1 2
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vn 0 0 -1
f 1 2 3
usemtl red
f 1/1/1 2/2/1 3/3/1 4/4/1
f 5/1 6/2 7/3 8/4
usemtl grey
f -5//1 -4//1 -3//1 -2//1 -1//1
usemtl nosuchmaterial
o part2
g group
s off
f 2 -12 1
f 1 2
"""


def restate(obj_text, mtl_text):
    """Independent reading of the same rules."""
    mats, by_name = [], {}
    for line in mtl_text.splitlines():
        t = line.split()
        if not t or t[0].startswith("#"):
            continue
        if t[0] == "newmtl":
            by_name[" ".join(t[1:])] = len(mats)
            mats.append([1.0, 1.0, 1.0, 1.0])
        elif t[0] == "Kd":
            v = [float(x) for x in t[1:4]]
            if len(v) == 1:
                v = v * 3
            mats[-1] = v + [1.0]
    pos, tcs, vi, ti, fm = [], [], [], [], []
    cur = -1
    for line in obj_text.splitlines():
        t = line.split()
        if not t or t[0].startswith("#"):
            continue
        if t[0] == "v":
            pos.append([float(x) for x in t[1:4]])
        elif t[0] == "vt":
            tcs.append([float(t[1]), float(t[2]) if len(t) > 2 else 0.0])
        elif t[0] == "usemtl":
            cur = by_name.get(" ".join(t[1:]), -1)
        elif t[0] == "f":
            cs = []
            for tok in t[1:]:
                parts = tok.split("/")
                v = int(parts[0])
                vt = int(parts[1]) if len(parts) > 1 and parts[1] else 0
                v = v - 1 if v > 0 else len(pos) + v
                vt = (vt - 1 if vt > 0 else len(tcs) + vt) if vt else -1
                cs.append((v, vt))
            if len(cs) < 3:
                continue
            if len(cs) == 3:
                tri = [0, 1, 2]
            elif len(cs) == 4:
                p = np.array([pos[c[0]] for c in cs], np.float32)
                d02 = np.float32(np.sum((p[2] - p[0]) ** 2, dtype=np.float32))
                d13 = np.float32(np.sum((p[3] - p[1]) ** 2, dtype=np.float32))
                tri = [0, 1, 2, 0, 2, 3] if d02 < d13 else [0, 1, 3, 1, 2, 3]
            else:
                tri = [k for j in range(1, len(cs) - 1) for k in (0, j, j + 1)]
            for k in tri:
                vi.append(cs[k][0])
                ti.append(cs[k][1] if cs[k][1] >= 0 else 0xFFFFFFFF)
            fm += [cur] * (len(tri) // 3)
    if any(m < 0 for m in fm):
        mats.append([1.0, 1.0, 1.0, 1.0])
    fm = [len(mats) - 1 if m < 0 else m for m in fm]
    return (np.array(pos, np.float32), np.array(tcs, np.float32), np.array(vi, np.uint32), np.array(ti, np.uint32),
            np.array(fm, np.uint32), np.array(mats, np.float32))


def run_parse(tmp_path):
    (tmp_path / "test.mtl").write_text(MTL)
    (tmp_path / "test.obj").write_text(OBJ)
    out = tmp_path / "out.bin"
    r = subprocess.run([EXE, "obj", str(tmp_path / "test.obj"), str(out)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    b = out.read_bytes()
    npos, ntc, ntri, nmat = np.frombuffer(b, np.uint32, 4)
    off = 16

    def take(dt, n):
        nonlocal off
        a = np.frombuffer(b, dt, n, off)
        off += a.nbytes
        return a

    pos = take(np.float32, npos * 3).reshape(-1, 3)
    tc = take(np.float32, ntc * 2).reshape(-1, 2)
    vi = take(np.uint32, ntri * 3)
    ti = take(np.uint32, ntri * 3)
    mi = take(np.uint32, ntri)
    col = take(np.float32, nmat * 4).reshape(-1, 4)
    return pos, tc, vi, ti, mi, col


def test_obj_reader_matches_restatement(tmp_path):
    got = run_parse(tmp_path)
    want = restate(OBJ, MTL)
    names = ("positions", "texcoords", "vertex_indices", "texture_indices", "material_indices", "colours")
    for name, g, w in zip(names, got, want):
        assert g.shape == w.shape, name
        assert np.array_equal(g, w), name


def test_obj_known_counts(tmp_path):
    pos, tc, vi, ti, mi, col = run_parse(tmp_path)
    # 1 triangle + 2 quads (2 each) + 1 pentagon (3) + 1 triangle; the 2-corner face is dropped
    assert len(vi) == 3 * 9 and len(pos) == 13 and len(tc) == 4
    # faces before any usemtl and after an unknown one take the default material appended last
    assert mi[0] == 2 and mi[-1] == 2 and np.array_equal(col[2], [1, 1, 1, 1])
    assert np.allclose(col[0], [0.8, 0.1, 0.1, 1.0]) and np.allclose(col[1], [0.5, 0.5, 0.5, 1.0])


def test_obj_missing_file_fails(tmp_path):
    r = subprocess.run([EXE, "obj", str(tmp_path / "none.obj"), str(tmp_path / "o.bin")], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 1 and "cannot open" in r.stderr


@pytest.mark.parametrize("bad", ["v 1 2\n", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2/x 3\n"])
def test_obj_malformed_records_fail(tmp_path, bad):
    (tmp_path / "bad.obj").write_text(bad)
    r = subprocess.run([EXE, "obj", str(tmp_path / "bad.obj"), str(tmp_path / "o.bin")], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 1 and "bad.obj:" in r.stderr
