"""Scene ingest (rtg_mesh_load, host only): OBJ and PLY files give the
vertex / triangle arrays of the reference's loaders + PrimitiveBuilder --
corners as new vertices, polygons as fans, triangles with an inf / NaN Wald
record dropped and the rest renumbered -- checked against a restatement
here that uses the oracle's TriAccel records for the validity test."""
import struct

import numpy as np
import pytest

from gridrt import lib


def _valid(oracle, v0, v1, v2):
    verts = np.array([v0, v1, v2], np.float32)
    acc = np.empty((1, 12), np.float32)
    oracle.lib().orc_triaccel_build(verts.ravel(), np.array([0, 1, 2], np.int32), 1, acc.ravel())
    words = acc[0, [1, 2, 3, 4, 5, 6, 8, 9, 10]]
    return bool(np.isfinite(words).all())


def _expect(oracle, pos, faces, per_triangle_vertices):
    """Reference semantics: OBJ (per_triangle_vertices=False) pushes each face
    corner once and fans over them; PLY pushes three vertices per fan triangle."""
    verts, tris, src = [], [], []
    for f, face in enumerate(faces):
        fan = [(face[0], face[k], face[k + 1]) for k in range(1, len(face) - 1)]
        if not per_triangle_vertices:
            s = len(verts)
            verts.extend(pos[c] for c in face)
            cand = [(s, s + k, s + k + 1) for k in range(1, len(face) - 1)]
        else:
            cand = []
            for a, b, c in fan:
                s = len(verts)
                verts.extend([pos[a], pos[b], pos[c]])
                cand.append((s, s + 1, s + 2))
        for a, b, c in cand:
            if _valid(oracle, verts[a], verts[b], verts[c]):
                tris.append((a, b, c))
                src.append(f)
    return (np.array(verts, np.float32).reshape(-1, 3), np.array(tris, np.int32).reshape(-1, 3),
            np.array(src, np.int64))


def _mesh(seed=3):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-1, 1, size=(40, 3)).astype(np.float32)
    pos[39] = pos[38] = pos[37]                      # a degenerate (zero-area) triangle below
    faces = [list(rng.choice(37, size=3, replace=False)) for _ in range(20)]
    faces += [list(rng.choice(37, size=4, replace=False)) for _ in range(6)]
    faces += [list(rng.choice(37, size=5, replace=False))]
    faces += [[37, 38, 39], [0, 1, 37]]
    return pos, faces


def test_obj_matches_reference_semantics(oracle, tmp_path):
    pos, faces = _mesh()
    p = tmp_path / "m.obj"
    with open(p, "w") as f:
        f.write("# test mesh\nvn 0 0 1\nvt 0 0\n")
        for v in pos:
            f.write(f"v {float(v[0])!r} {float(v[1])!r} {float(v[2])!r}\n")
        for j, face in enumerate(faces):
            toks = []
            for c in face:
                if j % 3 == 0:
                    toks.append(f"{c + 1}")
                elif j % 3 == 1:
                    toks.append(f"{c + 1}/1/1")
                else:
                    toks.append(f"{c - len(pos)}//1")    # negative: relative to the vertices so far
            f.write("f " + " ".join(toks) + "\n")
    verts, tris, src, info = lib.load_mesh(p)
    ev, et, es = _expect(oracle, pos, faces, per_triangle_vertices=False)
    assert np.array_equal(verts, ev) and np.array_equal(tris, et) and np.array_equal(src, es)
    assert info["faces"] == len(faces) and info["dropped"] == 1


def _write_ply(path, pos, faces, fmt):
    head = (f"ply\nformat {fmt} 1.0\ncomment test\nelement vertex {len(pos)}\nproperty float x\n"
            f"property float y\nproperty float z\nproperty uchar red\nelement face {len(faces)}\n"
            f"property list uchar int vertex_indices\nend_header\n")
    with open(path, "wb") as f:
        f.write(head.encode())
        if fmt == "ascii":
            for v in pos:
                f.write(f"{float(v[0])!r} {float(v[1])!r} {float(v[2])!r} 7\n".encode())
            for face in faces:
                f.write((f"{len(face)} " + " ".join(str(int(c)) for c in face) + "\n").encode())
        else:
            e = "<" if fmt == "binary_little_endian" else ">"
            for v in pos:
                f.write(struct.pack(e + "fffB", float(v[0]), float(v[1]), float(v[2]), 7))
            for face in faces:
                f.write(struct.pack(e + "B" + "i" * len(face), len(face), *[int(c) for c in face]))


@pytest.mark.parametrize("fmt", ["ascii", "binary_little_endian", "binary_big_endian"])
def test_ply_matches_reference_semantics(oracle, tmp_path, fmt):
    pos, faces = _mesh(5)
    p = tmp_path / "m.ply"
    _write_ply(p, pos, faces, fmt)
    verts, tris, src, info = lib.load_mesh(p)
    ev, et, es = _expect(oracle, pos, faces, per_triangle_vertices=True)
    assert np.array_equal(verts, ev) and np.array_equal(tris, et) and np.array_equal(src, es)
    assert info["dropped"] == 1


def test_bad_files(tmp_path):
    p = tmp_path / "bad.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nf 1 2 3\n")
    with pytest.raises(Exception):
        lib.load_mesh(p)
    q = tmp_path / "x.stl"
    q.write_text("solid")
    with pytest.raises(Exception):
        lib.load_mesh(q)
    with pytest.raises(Exception):
        lib.load_mesh(tmp_path / "missing.obj")
