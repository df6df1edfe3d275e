"""The library's model and image file loaders (host code, no GPU) against the
reference's own loadMesh / loadSTL / loadOBJ / X3D reader / loadPPM /
savePPM / saveSTL (src/io.cpp, src/x3d.cpp built into the oracle): the same
scene tree, bit-identical arrays and materials, identical written files.
Without the reference build the same models are checked against digests of
the reference's output (tests/golden/loaders.json, tests/golden/make_golden.py)."""
import ctypes as C
import hashlib
import json
import os
import struct

import numpy as np
import pytest

import loader_files
from minirender_gb300 import abi, capi, loaders
from minirender_gb300 import workloads as W
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "loaders.json")
MESH_KEYS = ("vertices", "normals", "texcoords", "indices", "normalsI", "texcoordsI")


@pytest.fixture(scope="module")
def files(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("models"))
    return d, loader_files.write_all(d)


def product_model(path):
    """The product's model as the oracle flattens the reference's: nodes,
    mesh arrays and textures decoded as loadPPM does (b / 255.0f)."""
    L = capi.lib()
    h = C.c_void_p()
    rc = L.mr_model_load(path.encode(), C.byref(h))
    if rc != 0:
        return None
    try:
        nn, nm, nt = C.c_int32(), C.c_int32(), C.c_int32()
        L.mr_model_counts(h, C.byref(nn), C.byref(nm), C.byref(nt))
        nodes = (abi.mr_node * max(1, nn.value))()
        assert L.mr_model_nodes(h, nodes, nn.value) == 0
        meshes = []
        for i in range(nm.value):
            d = abi.mr_mesh_desc()
            assert L.mr_model_mesh(h, i, C.byref(d)) == 0
            def arr(p, n, dt, cols):
                if n == 0:
                    return np.zeros((0, cols) if cols else 0, dt)
                ct = C.c_float if dt == np.float32 else C.c_int32
                a = np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), shape=(n * (cols or 1),)).copy()
                return a.reshape(-1, cols) if cols else a
            meshes.append({"vertices": arr(d.vertices, d.n_vertices, np.float32, 3),
                           "normals": arr(d.normals, d.n_normals, np.float32, 3),
                           "texcoords": arr(d.texcoords, d.n_texcoords, np.float32, 2),
                           "indices": arr(d.indices, d.n_indices, np.int32, 0),
                           "normalsI": arr(d.normalsI, d.n_normalsI, np.int32, 0),
                           "texcoordsI": arr(d.texcoordsI, d.n_texcoordsI, np.int32, 0)})
        textures = []
        for i in range(nt.value):
            p, r, c = C.POINTER(C.c_uint8)(), C.c_int32(), C.c_int32()
            assert L.mr_model_texture(h, i, C.byref(p), C.byref(r), C.byref(c)) == 0
            b = np.ctypeslib.as_array(p, shape=(r.value * c.value * 3,)).copy().reshape(r.value, c.value, 3)
            textures.append(b.astype(np.float32) / np.float32(255))
        return {"nodes": nodes[:nn.value], "meshes": meshes, "textures": textures}
    finally:
        L.mr_model_free(h)


def canonical(model):
    """Byte serialisation of a flattened model (texture indices replaced by
    the texture's pixels, so shared or duplicated textures compare equal)."""
    if model is None:
        return b"null"
    out = [struct.pack("<i", len(model["nodes"]))]
    for nd in model["nodes"]:
        out.append(struct.pack("<iii", nd.parent, nd.mesh, nd.has_material))
        out.append(np.array(nd.transform[:], np.float32).tobytes())
        if nd.has_material:
            m = nd.material
            out.append(np.array(list(m.diffuse) + list(m.specular) + list(m.emissive) + [m.shininess, nd.opacity],
                                np.float32).tobytes())
            t = model["textures"][m.texture] if m.texture >= 0 else None
            out.append(b"notex" if t is None else struct.pack("<ii", *t.shape[:2]) + t.astype(np.float32).tobytes())
    for m in model["meshes"]:
        for k in MESH_KEYS:
            out.append(k.encode() + struct.pack("<q", m[k].size) + np.ascontiguousarray(m[k]).tobytes())
    return b"".join(out)


def digest(model):
    return hashlib.sha256(canonical(model)).hexdigest()


def _golden():
    with open(GOLDEN) as f:
        return json.load(f)


# (digest key, writer) of the seeded random files whose reference digests
# tests/golden/make_golden.py records
RANDOM_FILES = ([(f"random_obj/{s}", lambda d, s=s: loader_files.random_obj(d, s)) for s in range(8)] +
                [(f"random_stl/{s}", lambda d, s=s: loader_files.random_ascii_stl(d, s)) for s in range(4)] +
                [(f"random_x3d/{s}", lambda d, s=s: loader_files.random_x3d(d, s)) for s in range(8)])


def test_models_match_golden(files, product_lib):
    d, names = files
    g = _golden()
    for n in names:
        assert digest(product_model(os.path.join(d, n))) == g[n], n


def test_models_match_reference(files, product_lib, ref_lib):
    d, names = files
    for n in names:
        p = os.path.join(d, n)
        ref = O.ref_load_mesh(p)
        got = product_model(p)
        assert (ref is None) == (got is None), n
        assert len(got["nodes"]) == len(ref["nodes"]), n
        for a, b in zip(got["nodes"], ref["nodes"]):
            assert (a.parent, a.mesh, a.has_material) == (b.parent, b.mesh, b.has_material), n
        for i, (a, b) in enumerate(zip(got["meshes"], ref["meshes"])):
            for k in MESH_KEYS:
                assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), (n, i, k)
        assert canonical(got) == canonical(ref), n


def test_python_scene_from_model(files, product_lib):
    """load_mesh builds the scene-model objects the renderer mirror takes."""
    d, names = files
    node = loaders.load_mesh(os.path.join(d, "parts.obj"))
    meshes = node.children
    assert [type(m).__name__ for m in meshes] == ["TriMesh"] * 4  # "", nosuch, red, wood
    wood = meshes[3]
    assert wood.material.texture is not None and wood.material.texture.shape == (16, 24, 3)
    assert np.isclose(float(meshes[2].material.shininess), 10.0)  # Ns 0 -> 10
    assert all(m.indices.size % 3 == 0 for m in meshes)
    x = loaders.load_mesh(os.path.join(d, "scene.x3d"))
    assert len(x.children) >= 3


def test_ppm_load_save_match_reference(tmp_path, product_lib, ref_lib):
    rng = np.random.default_rng(5)
    img = rng.integers(0, 256, (13, 29, 3)).astype(np.uint8)
    p = str(tmp_path / "a.ppm")
    loader_files._ppm(p, img, comment=True)
    got = loaders.load_ppm(p)
    assert np.array_equal(got, img)
    assert np.array_equal((got.astype(np.float32) / np.float32(255)).view(np.uint32),
                          O.ref_load_ppm(p).view(np.uint32))
    # savePPM: the reference quantises floats; the library writes the bytes the device produced
    f = rng.uniform(-0.2, 1.2, (7, 11, 3)).astype(np.float32)
    q = O.quantize_rgb8(f)
    a, b = str(tmp_path / "ref.ppm"), str(tmp_path / "gpu.ppm")
    O.ref_save_ppm(a, f)
    loaders.save_ppm(b, q)
    assert open(a, "rb").read() == open(b, "rb").read()


def test_stl_save_matches_reference(tmp_path, product_lib, ref_lib):
    st, sc = W.config1(64, 48)
    m = sc.children[0]
    xf = np.array([[0.5, 0, 0.1, 1], [0, 2, 0, -1], [0.3, 0, 1, 0.25], [0, 0, 0, 1]], np.float32)
    a, b = str(tmp_path / "ref.stl"), str(tmp_path / "gpu.stl")
    O.ref_save_stl(a, m.desc(), xf)
    loaders.save_stl(b, m, xf)
    assert open(a, "rb").read() == open(b, "rb").read()


def test_xyz_save_matches_reference(tmp_path, product_lib, ref_lib):
    """saveXYZ of a range image and of points around the z < -1e-5 cut,
    with the identity and with a transform: the same text as the
    reference's own saveXYZ."""
    st, sc = W.config1(64, 48)
    rng_img = O.range_image(st, O.render(st, sc)["depth"])
    rng = np.random.default_rng(12)
    pts = rng.normal(size=(9, 13, 3)).astype(np.float32)
    pts[0, :4, 2] = np.float32([-1e-5, -1.0001e-5, 0.0, -0.0])  # exactly at, just past, zero, negative zero
    xf = np.array([[0.5, 0, 0.1, 1], [0, 2, 0, -1], [0.3, 0, 1, 0.25], [0, 0, 0, 1]], np.float32)
    for k, (img, m) in enumerate([(rng_img, None), (rng_img, xf), (pts, None), (pts, xf)]):
        a, b = str(tmp_path / f"ref{k}.xyz"), str(tmp_path / f"gpu{k}.xyz")
        O.ref_save_xyz(a, img, m)
        loaders.save_xyz(b, img, m)
        assert open(a, "rb").read() == open(b, "rb").read(), k
    assert len(open(str(tmp_path / "gpu0.xyz")).read().splitlines()) == int((rng_img[..., 2] < -1e-5).sum()) > 100


def test_xyz_save_rejects_bad_arguments(tmp_path, product_lib):
    L = capi.lib()
    p = str(tmp_path / "x.xyz").encode()
    assert L.mr_xyz_save(None, None, 0, 0, None) == abi.MR_E_INVALID
    assert L.mr_xyz_save(p, None, -1, 3, None) == abi.MR_E_INVALID
    assert L.mr_xyz_save(p, None, 2, 3, None) == abi.MR_E_INVALID
    assert L.mr_xyz_save(p, None, 0, 3, None) == abi.MR_OK  # empty image, empty file
    assert os.path.getsize(p.decode()) == 0


def test_large_files_parsed_in_parallel_match_reference(tmp_path, product_lib, ref_lib):
    """Binary STL above 200k facets and OBJ above 4 MB take the multi-threaded
    paths; the result is the same as the reference's serial parse."""
    rng = np.random.default_rng(8)
    nf = 250_000
    p = str(tmp_path / "big.stl")
    rec = np.zeros(nf, dtype=[("f", "<f4", 12), ("a", "<i2")])
    rec["f"] = rng.normal(size=(nf, 12)).astype(np.float32)
    with open(p, "wb") as f:
        f.write(b" " * 80 + struct.pack("<i", nf) + rec.tobytes())
    assert canonical(product_model(p)) == canonical(O.ref_load_mesh(p))
    q = str(tmp_path / "big.obj")
    nv = 60_000
    with open(q, "w") as f:
        for v in rng.uniform(-1, 1, (nv, 3)).astype(np.float32):
            f.write("v %r %r %r\n" % tuple(float(x) for x in v))
        for v in rng.normal(size=(nv, 3)).astype(np.float32):
            f.write("vn %r %r %r\n" % tuple(float(x) for x in v))
        for k in range(60_000):
            ids = rng.choice(nv, 3 + k % 2, replace=False) + 1
            f.write("f " + " ".join(f"{i}//{i}" for i in ids) + "\n")
    assert os.path.getsize(q) > 4 << 20
    assert canonical(product_model(q)) == canonical(O.ref_load_mesh(q))


def test_errors(tmp_path, product_lib):
    L = capi.lib()
    h = C.c_void_p()
    assert L.mr_model_load(str(tmp_path / "missing.stl").encode(), C.byref(h)) == abi.MR_E_IO
    bad = tmp_path / "bad.stl"
    bad.write_bytes(b"nothing like an stl file here\n")
    assert L.mr_model_load(str(bad).encode(), C.byref(h)) == abi.MR_E_IO
    nx = tmp_path / "notx3d.x3d"
    nx.write_text("<html><body/></html>")
    assert L.mr_model_load(str(nx).encode(), C.byref(h)) == abi.MR_E_IO
    other = tmp_path / "model.xyz"
    other.write_text("1 2 3\n")
    node = loaders.load_mesh(str(other))  # loadMesh: an empty node for other extensions
    assert node.children == []
    with pytest.raises(capi.MRError):
        loaders.load_ppm(str(bad))


@pytest.mark.parametrize("seed", range(32))
def test_random_obj_matches_reference(tmp_path, product_lib, ref_lib, seed):
    """Seeded random OBJ + MTL files (tests/loader_files.random_obj): the
    same scene tree, arrays and materials as the reference's loadOBJ."""
    name = loader_files.random_obj(str(tmp_path), seed)
    p = str(tmp_path / name)
    ref = O.ref_load_mesh(p)
    got = product_model(p)
    assert ref is not None and got is not None
    assert canonical(got) == canonical(ref)


@pytest.mark.parametrize("seed", range(16))
def test_random_ascii_stl_matches_reference(tmp_path, product_lib, ref_lib, seed):
    """Seeded random ASCII STL files: the same mesh as the reference's loadSTLa."""
    name = loader_files.random_ascii_stl(str(tmp_path), seed)
    p = str(tmp_path / name)
    ref = O.ref_load_mesh(p)
    got = product_model(p)
    assert ref is not None and got is not None
    assert canonical(got) == canonical(ref)


@pytest.mark.parametrize("seed", range(32))
def test_random_x3d_matches_reference(tmp_path, product_lib, ref_lib, seed):
    """Seeded random X3D scenes (tests/loader_files.random_x3d): the same
    scene tree, transforms, arrays and materials as the reference's reader."""
    name = loader_files.random_x3d(str(tmp_path), seed)
    p = str(tmp_path / name)
    ref = O.ref_load_mesh(p)
    got = product_model(p)
    assert ref is not None and got is not None
    assert canonical(got) == canonical(ref)


def test_mutated_files_never_crash(tmp_path, product_lib):
    """Truncated, byte-flipped, spliced and token-injected copies of every
    sample and random file load or fail with a status, never crash; a model
    that loads reports consistent counts (the reference has no such checks:
    its loaders index past the ends of short lines and lists)."""
    d = str(tmp_path)
    names = loader_files.write_all(d)
    for s in range(4):
        names += [loader_files.random_obj(d, s), loader_files.random_x3d(d, s), loader_files.random_ascii_stl(d, s)]
    toks = [b"-1", b" ", b"/", b"//", b"f", b"v", b"\n", b"<", b">", b"'", b'"', b'USE="C0"', b"99999",
            b"-99999", b"nan", b"1e40", b"\x00"]
    rng = np.random.default_rng(3)
    L = capi.lib()
    loaded = 0
    for it in range(600):
        n = names[int(rng.integers(len(names)))]
        data = bytearray(open(os.path.join(d, n), "rb").read())
        k = it % 4
        if k == 0:
            data = data[:int(rng.integers(len(data)))]
        elif k == 1:
            for _ in range(int(rng.integers(1, 20))):
                data[int(rng.integers(len(data)))] = int(rng.integers(256))
        elif k == 2:
            pos = int(rng.integers(len(data) + 1))
            data = data[:pos] + toks[int(rng.integers(len(toks)))] + data[pos:]
        else:
            a, b = sorted(int(x) for x in rng.integers(0, len(data) + 1, 2))
            data = data[:a] + data[b:]
        p = os.path.join(d, "mut_" + n)
        with open(p, "wb") as f:
            f.write(bytes(data))
        h = C.c_void_p()
        rc = L.mr_model_load(p.encode(), C.byref(h))
        if rc == 0:
            nn, nm, nt = C.c_int32(), C.c_int32(), C.c_int32()
            assert L.mr_model_counts(h, C.byref(nn), C.byref(nm), C.byref(nt)) == 0
            assert nn.value >= 1 and nm.value >= 0 and nt.value >= 0
            L.mr_model_free(h)
            loaded += 1
        else:
            assert rc in (abi.MR_E_IO, abi.MR_E_INVALID, abi.MR_E_NOMEM), (n, k, rc)
    assert loaded > 100


@pytest.mark.parametrize("key", [k for k, _ in RANDOM_FILES])
def test_random_models_match_golden(tmp_path, product_lib, key):
    """Seeded random files against digests of the reference loaders' output
    (no reference build needed)."""
    make = dict(RANDOM_FILES)[key]
    name = make(str(tmp_path))
    assert digest(product_model(str(tmp_path / name))) == _golden()[key]
