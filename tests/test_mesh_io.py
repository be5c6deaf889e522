"""Model and texture ingest (ct_mesh_load_obj, ct_image_load) and the
TriangleList.load_model mirror of TriangleList::loadModel
(src/Core/TriangleList.cpp:63-146, 203-348). Host only: procedural OBJ/MTL/TGA
files with hand-derived expectations, plus the reference's own models where
its tree is present."""
import os
import struct

import numpy as np
import pytest

from cudatracer_gb300 import _lib, api


def _write(path, text):
    with open(path, "w") as f:
        f.write(text)
    return str(path)


def test_polygon_split_winding_and_joined_vertices(lib, tmp_path):
    obj = _write(tmp_path / "poly.obj", """
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 2 0 0
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vn 0 0 1
f 1/1/1 2/2/1 3/3/1 4/4/1
f 2/2/1 5/2/1 3/3/1
f -5/1/1 -4/2/1 -3/3/1
""")
    m = api.load_obj(obj, normalize=False)
    # quad (1,2,3,4) reversed to (4,3,2,1) and fanned: (4,3,2), (4,2,1)
    p = m["vertices"][m["indices"]]
    expect = np.array([[[0, 1, 0], [1, 1, 0], [1, 0, 0]],
                       [[0, 1, 0], [1, 0, 0], [0, 0, 0]],
                       [[1, 1, 0], [2, 0, 0], [1, 0, 0]],
                       [[1, 1, 0], [1, 0, 0], [0, 0, 0]]], np.float32)
    assert np.array_equal(p, expect)
    # corners (v,t,n) are joined: 4 from the quad + vertex 5 with texcoord 2
    assert m["vertices"].shape == (5, 3)
    assert np.array_equal(m["texcoords"][m["indices"][1]], np.array([[0, 1], [1, 0], [0, 0]], np.float32))
    assert (m["normals"] == np.array([0, 0, 1], np.float32)).all()
    assert (m["material_idxs"] == 0).all() and len(m["materials"]) == 1


def test_missing_texcoords_and_generated_normals(lib, tmp_path):
    # an octahedron without normals or texcoords, faces counter-clockwise seen from outside
    v = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
    faces = [(0, 2, 4), (2, 1, 4), (1, 3, 4), (3, 0, 4), (2, 0, 5), (1, 2, 5), (3, 1, 5), (0, 3, 5)]
    text = "".join(f"v {x} {y} {z}\n" for x, y, z in v) + "".join(f"f {a+1} {b+1} {c+1}\n" for a, b, c in faces)
    m = api.load_obj(_write(tmp_path / "oct.obj", text), normalize=False)
    assert m["indices"].shape == (8, 3) and m["vertices"].shape == (6, 3)
    # smooth normals point out along the vertex direction
    assert np.allclose(m["normals"], m["vertices"], atol=1e-6)
    assert (m["texcoords"] == 0.5).all()
    # stored winding is reversed: the right-hand normal of each stored triangle points inward
    t = m["vertices"][m["indices"]]
    n = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    assert (np.einsum("ij,ij->i", n, t.mean(axis=1)) < 0).all()


def test_normalize_centres_and_scales(lib, tmp_path):
    text = "v 10 20 30\nv 14 20 30\nv 10 21 32\nf 1 2 3\n"
    m = api.load_obj(_write(tmp_path / "t.obj", text), normalize=True)
    lo, hi = m["vertices"].min(0), m["vertices"].max(0)
    assert np.allclose(lo + hi, 0, atol=1e-6)
    assert np.isclose((hi - lo).max(), 2.0)
    assert np.allclose(hi - lo, [2.0, 0.5, 1.0])


MTL = """
newmtl textured
Kd 0.5 0.5 0.5
Ns 7.8
map_Kd tex/a.tga
newmtl textured_dull
Ns 1.5
map_Kd -bm 1 tex/a.tga
newmtl lamp
Kd 0 0 0
Ke 4 5 0.001
newmtl paint
Kd 0.2 0.3 0.4
Ks 0.5 0.5 0.5
Ns 0
newmtl glossy
Kd 0.5 0.4 0.3
Ns 20
newmtl mirror
Kd 0 0 0
Ks 0.9 0.8 0.7
newmtl glass
Kd 0 0 0
Tf 0.9 0.95 1
Ni 1.45
newmtl rough_glass
Kd 0 0 0
Tf 0.9 0.95 1
Ns 10
newmtl black
Kd 0 0 0
Tf 0 0 0
newmtl bumpy
Kd 0.5 0.5 0.5
norm tex/n.tga
"""


def test_material_choice_follows_process_mesh(lib, tmp_path):
    _write(tmp_path / "m.mtl", MTL)
    names = ["textured", "textured_dull", "lamp", "paint", "glossy", "mirror", "glass", "rough_glass", "black",
             "bumpy", "not_in_library"]
    text = "mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n"
    text += "".join(f"usemtl {n}\nf 1 2 3\n" for n in names)
    m = api.load_obj(_write(tmp_path / "mats.obj", text), normalize=False)
    mats = m["materials"]
    # faces before any usemtl use the importer's default material (diffuse 0.6 grey)
    assert len(mats) == len(names) + 1
    assert list(m["material_idxs"]) == list(range(len(names) + 1))
    d = {n: mats[i + 1] for i, n in enumerate(names)}
    dflt = mats[0]
    assert dflt.type == api.MAT_LAMBERTIAN and np.allclose(dflt.albedo, 0.6)
    assert d["textured"].type == api.MAT_GGX and d["textured"].albedo == (1.0, 1.0, 1.0)
    assert np.isclose(d["textured"].roughness, 7.8)
    assert m["diffuse_maps"][1] == str(tmp_path / "tex/a.tga")
    assert d["textured_dull"].type == api.MAT_LAMBERTIAN and m["diffuse_maps"][2] == str(tmp_path / "tex/a.tga")
    assert d["lamp"].type == api.MAT_LIGHT and np.allclose(d["lamp"].albedo, [4, 5, 0.01])
    # the specular colour wins when it is the brighter one
    assert d["paint"].type == api.MAT_LAMBERTIAN and np.allclose(d["paint"].albedo, 0.5)
    assert d["glossy"].type == api.MAT_GGX and np.allclose(d["glossy"].albedo, [0.5, 0.4, 0.3])
    assert d["mirror"].type == api.MAT_SPECULAR and np.allclose(d["mirror"].albedo, [0.9, 0.8, 0.7])
    assert np.isclose(d["mirror"].refract_idx, 1.0)
    g = d["glass"]
    assert g.type == api.MAT_FRESNEL and np.isclose(g.refract_idx, 1.45)
    assert np.allclose(g.absorption, [0.9, 0.95, 1]) and np.allclose(g.albedo, [0.9, 0.95, 1])
    assert d["rough_glass"].type == api.MAT_FRESNEL_GGX and np.isclose(d["rough_glass"].refract_idx, 1.0)
    assert d["black"].type == api.MAT_LAMBERTIAN and d["black"].albedo == (0.0, 0.0, 0.0)
    assert m["normal_maps"][10] == str(tmp_path / "tex/n.tga")
    assert all(x.diffuse_tex == -1 and x.normal_tex == -1 for x in mats)


@pytest.mark.parametrize("text,what", [
    ("v 0 0 0\nv 1 0 0\nf 1 2 4\n", "index out of range"),
    ("v 0 0 0\nv 1 0 0\nf 1 2\n", "two corners"),
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1/x 2 3\n", "not a number"),
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 0 2 3\n", "index zero"),
    ("v 0 0 0\n", "no faces"),
])
def test_bad_files_fail_with_a_message(lib, tmp_path, text, what):
    with pytest.raises(_lib.CTError) as e:
        api.load_obj(_write(tmp_path / "bad.obj", text))
    assert e.value.status == _lib.CT_ERR_INVALID_ARGUMENT
    assert str(tmp_path) in str(e.value) or "line" in str(e.value) or "corner" in str(e.value)


def test_missing_file(lib, tmp_path):
    with pytest.raises(_lib.CTError):
        api.load_obj(str(tmp_path / "nope.obj"))
    with pytest.raises(_lib.CTError):
        api.load_image(str(tmp_path / "nope.tga"))


def _tga(path, img, kind="rgb", top_first=False, rle=False, right_first=False):
    """Write an (h, w, 3|1) uint8 image (row 0 = top of the picture)."""
    h, w = img.shape[:2]
    rows = img if top_first else img[::-1]
    if right_first:
        rows = rows[:, ::-1]
    if kind == "rgb":
        px = [bytes(p[::-1]) for p in rows.reshape(-1, 3)]  # BGR
        base, bpp = 2, 24
    elif kind == "rgba":
        px = [bytes(list(p[::-1]) + [255]) for p in rows.reshape(-1, 3)]
        base, bpp = 2, 32
    elif kind == "grey":
        px = [bytes([p]) for p in rows.reshape(-1)]
        base, bpp = 3, 8
    elif kind == "mapped":
        pal = sorted({tuple(p) for p in rows.reshape(-1, 3)})
        px = [bytes([pal.index(tuple(p))]) for p in rows.reshape(-1, 3)]
        base, bpp = 1, 8
    desc = (0x20 if top_first else 0) | (0x10 if right_first else 0) | (8 if kind == "rgba" else 0)
    cmap = b""
    head_cmap = (0, 0, 0, 0)
    if kind == "mapped":
        cmap = b"".join(bytes(p[::-1]) for p in pal)
        head_cmap = (1, 0, len(pal), 24)
    data = b""
    if not rle:
        data = b"".join(px)
    else:
        i = 0
        while i < len(px):
            j = i
            while j + 1 < len(px) and px[j + 1] == px[i] and j - i < 127:
                j += 1
            if j > i:
                data += bytes([0x80 | (j - i)]) + px[i]
                i = j + 1
            else:
                k = i
                while k + 1 < len(px) and px[k + 1] != px[k] and k - i < 127:
                    k += 1
                if k + 1 < len(px) and px[k + 1] == px[k] and k > i:
                    k -= 1
                data += bytes([k - i]) + b"".join(px[i:k + 1])
                i = k + 1
    head = struct.pack("<BBBHHBHHHHBB", 0, head_cmap[0], base + (8 if rle else 0), head_cmap[1], head_cmap[2],
                       head_cmap[3], 0, 0, w, h, bpp, desc)
    with open(path, "wb") as f:
        f.write(head + cmap + data)
    return str(path)


@pytest.mark.parametrize("kind,top_first,rle,right_first", [
    ("rgb", False, False, False), ("rgb", True, False, False), ("rgba", True, True, False),
    ("rgb", False, True, True), ("grey", False, False, False), ("grey", True, True, False),
    ("mapped", False, False, False), ("mapped", True, True, False)])
def test_tga_matches_surface_layout(lib, tmp_path, kind, top_first, rle, right_first):
    rng = np.random.default_rng(3)
    h, w = 7, 5
    if kind == "grey":
        g = rng.integers(0, 256, (h, w), dtype=np.uint8)
        g[2, :] = 9  # a run for the RLE encoder
        img3 = np.repeat(g[..., None], 3, axis=2)
        src = g
    else:
        img3 = rng.integers(0, 4 if kind == "mapped" else 256, (h, w, 3), dtype=np.uint8) * (60 if kind == "mapped" else 1)
        img3[3, :] = (10, 20, 30)
        src = img3
    p = _tga(tmp_path / "t.tga", src, kind, top_first, rle, right_first)
    t = api.load_image(p)
    assert t.shape == (h, w, 4)
    # row 0 is the bottom of the picture; channel / 255; alpha 1
    expect = img3[::-1].astype(np.float32) / np.float32(255.0)
    assert np.array_equal(t[..., :3], expect)
    assert (t[..., 3] == 1.0).all()


def test_truncated_tga_fails(lib, tmp_path):
    p = _tga(tmp_path / "t.tga", np.zeros((4, 4, 3), np.uint8))
    with open(p, "rb") as f:
        b = f.read()
    with open(p, "wb") as f:
        f.write(b[:-5])
    with pytest.raises(_lib.CTError):
        api.load_image(p)


def test_load_model_transforms_materials_and_textures(lib, tmp_path):
    os.makedirs(tmp_path / "tex")
    _tga(tmp_path / "tex/a.tga", np.full((2, 3, 3), 200, np.uint8))
    _write(tmp_path / "m.mtl", MTL)
    text = ("mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nv 0 0 1\nvn 0 0 1\n"
            "usemtl textured\nf 1//1 2//1 3//1\nusemtl lamp\nf 1//1 3//1 4//1\nusemtl textured_dull\nf 2//1 3//1 4//1\n")
    obj = _write(tmp_path / "s.obj", text)
    tl = api.TriangleList()
    M = np.eye(4, dtype=np.float32)
    M[:3, 3] = (5, 6, 7)
    M[0, 0] = 2.0
    imported = tl.load_model(obj, scale=0.5, mat=M.T.reshape(-1).reshape(4, 4).T, normalize=False)
    a = tl.arrays()
    # materials: the default one plus one per used MTL entry, roughness set to 1 as addMaterial does
    assert len(tl.materials) == 4 and all(m.roughness == 1.0 for m in tl.materials)
    assert [m.type for m in tl.materials[1:]] == [api.MAT_GGX, api.MAT_LIGHT, api.MAT_LAMBERTIAN]
    # both textured materials share the one texture
    assert tl.materials[1].diffuse_tex == 0 and tl.materials[3].diffuse_tex == 0 and len(tl.textures) == 1
    assert np.allclose(tl.textures[0], 200 / 255.0) or np.allclose(tl.textures[0][..., :3], np.float32(200) / 255)
    assert list(a["material_idxs"]) == [1, 2, 3]
    assert list(a["light_indices"]) == [1]
    # pos = M * (p * scale, 1)
    p = imported["vertices"] * 0.5
    expect = p * np.array([2, 1, 1], np.float32) + np.array([5, 6, 7], np.float32)
    assert np.allclose(a["vertices"], expect)
    # normals get M's rotation/scale but no translation (w = 0), not renormalised
    assert np.allclose(a["normals"], [0, 0, 1])
    # an explicit material overrides the file's
    tl2 = api.TriangleList()
    tl2.load_model(obj, material=0, normalize=False)
    assert (tl2.arrays()["material_idxs"] == 0).all() and tl2.arrays()["light_indices"].size == 0


def _reference_models():
    import ref_build

    d = os.path.join(os.environ.get("CT_REFERENCE_DIR", ref_build.DEFAULT_REFERENCE), "Models")
    if not os.path.isdir(d):
        pytest.skip("reference models not present")
    return d


def test_reference_models_import(lib):
    d = _reference_models()
    s = api.load_obj(os.path.join(d, "sphere.obj"))
    assert s["indices"].shape[0] == 960
    r = np.linalg.norm(s["vertices"], axis=1)
    assert r.max() <= 1.0 + 1e-5 and r.min() > 0.95
    # normals point outward on the unit sphere
    assert (np.einsum("ij,ij->i", s["normals"], s["vertices"]) > 0.9 * r).all()
    g = api.load_obj(os.path.join(d, "dragon.obj"))
    assert g["indices"].shape[0] == 46540
    ext = g["vertices"].max(0) - g["vertices"].min(0)
    assert np.isclose(ext.max(), 2.0, atol=1e-5)
    assert np.allclose(np.linalg.norm(g["normals"], axis=1), 1.0, atol=1e-5)


def test_reference_sponza_materials(lib, tmp_path):
    """The Sponza MTL through processMesh: every entry with a diffuse map and
    Ns 7.84 becomes a white GGX with that map."""
    d = os.path.join(_reference_models(), "sponza")
    names = []
    with open(os.path.join(d, "sponza.mtl")) as f:
        names = [ln.split()[1] for ln in f if ln.startswith("newmtl")]
    text = f"mtllib {os.path.join(d, 'sponza.mtl')}\nv 0 0 0\nv 1 0 0\nv 0 1 0\n"
    text += "".join(f"usemtl {n}\nf 1 2 3\n" for n in names)
    # mtllib paths are taken relative to the OBJ's folder
    obj = _write(os.path.join(tmp_path, "s.obj"), text.replace(os.path.join(d, "sponza.mtl"),
                                                               os.path.relpath(os.path.join(d, "sponza.mtl"), tmp_path)))
    os.symlink(os.path.join(d, "textures"), os.path.join(tmp_path, "textures"))  # maps resolve beside the OBJ
    m = api.load_obj(obj, normalize=False)
    assert len(m["materials"]) == len(names) == 25
    textured = [i for i, p in enumerate(m["diffuse_maps"]) if p]
    assert len(textured) == 24
    for i in textured:
        assert m["materials"][i].type == api.MAT_GGX and m["materials"][i].albedo == (1.0, 1.0, 1.0)
        assert m["diffuse_maps"][i].endswith(".tga")
    present = [m["diffuse_maps"][i] for i in textured if os.path.exists(m["diffuse_maps"][i])]
    assert present  # the tree ships only some of the maps its MTL names
    t = api.load_image(present[0])
    assert t.ndim == 3 and t.shape[2] == 4 and (t[..., 3] == 1).all() and 0 <= t.min() and t.max() <= 1
