"""SMD meshes (Mesh::LoadFromFile, src/s3d_mesh.cpp:250-465) and instancing by transform.

The loader reads files this test writes with the format's own layout (all five material
types, texture names, negative material ids), rejects damaged files, and -- where the
reference project is present -- loads the meshes it ships.  No GPU is needed.
"""
import os
import struct

import numpy as np
import pytest


def write_smd(path, pos, nrm, uv, mat_ids, materials, textures=(), version=2, magic=b"SMD\0"):
    """materials: (smd_type, dict) with the fields of that type."""
    with open(path, "wb") as f:
        f.write(magic)
        f.write(struct.pack("<II", version, 24))
        f.write(struct.pack("<6I", len(mat_ids), len(materials), len(textures), 100, 0, 256))
        for t in textures:
            f.write(t.encode().ljust(256, b"\0"))
        for kind, m in materials:
            f.write(struct.pack("<i", kind))
            if kind in (0, 1):
                f.write(struct.pack("<3f3fi", *m["color"], *m["emission"], m.get("map", -1)))
            elif kind == 2:
                f.write(struct.pack("<3ff3fi", *m["color"], m["ior"], *m["emission"], m.get("map", -1)))
            elif kind == 3:
                f.write(struct.pack("<3ff3fi", *m["color"], m["power"], *m["emission"], m.get("map", -1)))
            else:
                f.write(struct.pack("<3f3ff3fii", *m["diffuse"], *m["specular"], m["power"], *m["emission"],
                                    m.get("map", -1), -1))
        for t in range(len(mat_ids)):
            for k in range(3):
                f.write(struct.pack("<3f3f2f", *pos[t, 3 * k:3 * k + 3], *nrm[t, 3 * k:3 * k + 3], *uv[t, 2 * k:2 * k + 2]))
            f.write(struct.pack("<i", int(mat_ids[t])))


MATS = [(0, {"color": (0.7, 0.6, 0.5), "emission": (0, 0, 0), "map": 1}),
        (1, {"color": (0.9, 0.9, 0.9), "emission": (0, 0, 0)}),
        (2, {"color": (1.0, 1.0, 1.0), "ior": 1.33, "emission": (0, 0, 0)}),
        (3, {"color": (0.8, 0.7, 0.6), "power": 50.0, "emission": (0.5, 0, 0)}),
        (4, {"diffuse": (0.2, 0.3, 0.4), "specular": (0.5, 0.5, 0.5), "power": 200.0, "emission": (0, 0, 0)})]


def _mesh(n, seed=1):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-1, 1, (n, 9)).astype(np.float32)
    nrm = rng.normal(size=(n, 9)).astype(np.float32)
    uv = rng.uniform(0, 1, (n, 6)).astype(np.float32)
    ids = rng.integers(0, len(MATS), n).astype(np.int32)
    return pos, nrm, uv, ids


def test_loads_every_material_type(salty_lib, tmp_path):
    import salty_gb300
    pos, nrm, uv, ids = _mesh(257)
    ids[3] = -1  # no material: the reference passes null, the flat scene uses material 0
    p = str(tmp_path / "m.smd")
    write_smd(p, pos, nrm, uv, ids, MATS, textures=("a.bmp", "b.bmp"))
    m = salty_gb300.load_smd(p)
    np.testing.assert_array_equal(m["tri_pos"], pos)
    np.testing.assert_array_equal(m["tri_nrm"], nrm)
    np.testing.assert_array_equal(m["tri_uv"], uv)
    want = ids.copy()
    want[3] = 0
    np.testing.assert_array_equal(m["tri_mat"], want)
    types = [x["type"] for x in m["materials"]]
    assert types == [salty_gb300.LAMBERT, salty_gb300.MIRROR, salty_gb300.GLASS, salty_gb300.PHONG,
                     salty_gb300.PLASTIC]
    assert m["materials"][2]["ior"] == pytest.approx(1.33)
    assert m["materials"][3]["power"] == 50.0 and m["materials"][3]["emission"][0] == 0.5
    assert m["materials"][4]["specular"] == pytest.approx((0.5, 0.5, 0.5))
    assert m["materials"][4]["color"] == pytest.approx((0.2, 0.3, 0.4))
    assert m["textures"] == ["a.bmp", "b.bmp"] and m["mat_texture"] == [1, -1, -1, -1, -1]


@pytest.mark.parametrize("damage", ["magic", "version", "truncated", "material_index", "no_triangles"])
def test_rejects_damaged_files(salty_lib, tmp_path, damage):
    import salty_gb300
    pos, nrm, uv, ids = _mesh(10)
    p = str(tmp_path / "bad.smd")
    kw = {}
    if damage == "magic":
        kw["magic"] = b"OBJ\0"
    if damage == "version":
        kw["version"] = 1
    if damage == "material_index":
        ids[4] = len(MATS)
    if damage == "no_triangles":
        pos, nrm, uv, ids = pos[:0], nrm[:0], uv[:0], ids[:0]
    write_smd(p, pos, nrm, uv, ids, MATS, **kw)
    if damage == "truncated":
        with open(p, "r+b") as f:
            f.truncate(os.path.getsize(p) - 37)
    with pytest.raises(salty_gb300.SaltyError):
        salty_gb300.load_smd(p)


def test_reference_meshes_load(salty_lib):
    """The meshes the reference project ships (only where its sources are present)."""
    import salty_gb300
    from oracle.oracle import reference_dir
    root = reference_dir()
    if root is None:
        pytest.skip("reference sources not present here")
    for name, n in (("paper_cup", 1880), ("dosei", 19328)):
        p = os.path.join(root, "project", "res", "mesh", name, f"{name}.smd")
        if not os.path.exists(p):
            pytest.skip(f"{name}.smd not present")
        m = salty_gb300.load_smd(p)
        assert m["tri_pos"].shape == (n, 9)
        assert np.all(np.isfinite(m["tri_pos"])) and np.all(np.isfinite(m["tri_nrm"]))
        assert m["tri_mat"].min() >= 0 and m["tri_mat"].max() < len(m["materials"])


def test_transform_places_positions_and_normals(salty_lib):
    import salty_gb300
    pos, nrm, _, _ = _mesh(50, seed=3)
    nrm /= np.linalg.norm(nrm.reshape(-1, 3), axis=1).reshape(50, 3).repeat(3, axis=1)
    rng = np.random.default_rng(4)
    A = rng.normal(size=(3, 3))
    t = rng.normal(size=3)
    M = np.concatenate([A, t[:, None]], axis=1)
    p2, n2 = salty_gb300.transform_mesh(M, pos, nrm)
    P = pos.reshape(-1, 3).astype(np.float64)
    np.testing.assert_allclose(p2.reshape(-1, 3), P @ A.T + t, rtol=1e-5, atol=1e-5)
    want = nrm.reshape(-1, 3).astype(np.float64) @ np.linalg.inv(A)
    want /= np.linalg.norm(want, axis=1, keepdims=True)
    np.testing.assert_allclose(n2.reshape(-1, 3), want, rtol=1e-5, atol=1e-5)
    with pytest.raises(salty_gb300.SaltyError):
        salty_gb300.transform_mesh(np.zeros((3, 4)), pos)
