"""The C++ binding a maintainer adds beside the reference's Renderer
(minirender_gb300/cpp/GpuRenderer.*: Renderer's public methods over the C
ABI), built and run through a small driver (tests/cpp/binding_main.cpp).

CPU: the binding and the driver compile and link against the library, with
the reference's own Scene.h and Scene.cpp where the reference sources are
present and with the scene-model stand-in of tests/cpp everywhere; without
a GPU the binding reports MR_E_NO_DEVICE through GpuError (no CPU path).

GPU: frames rendered through GpuRenderer -- the 640x480 sphere, models read
by the library's loaders (OBJ with a texture, X3D with transforms), random
scenes with normals saved, and render() followed by paintMesh /
paintTriangle runs -- equal the oracle's (ids and depth bit for bit, RGB8
within 1 LSB on >= 99.9 % of pixels); getRangeImage equals the oracle's
range image bit for bit."""
import os
import subprocess

import numpy as np
import pytest

from minirender_gb300 import abi, build
from minirender_gb300 import scene as S
from minirender_gb300 import workloads as W
from oracle import oracle as O
from parity import assert_parity, compare

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "minirender_gb300", "cpp")
TCPP = os.path.join(ROOT, "tests", "cpp")
SHIM = os.path.join(ROOT, "oracle", "asl_shim")


def build_driver(out_dir: str, against_reference: bool = False) -> str:
    """g++ build of the driver and the binding; the scene model is the
    reference's (headers and Scene.cpp, read in place) or the stand-in."""
    lib = build.build()
    lib_dir = os.path.dirname(lib)
    exe = os.path.join(out_dir, "binding_main_ref" if against_reference else "binding_main")
    inc = ["-I", CPP, "-I", os.path.join(ROOT, "include"), "-I", SHIM]
    srcs = [os.path.join(CPP, "GpuRenderer.cpp"), os.path.join(TCPP, "binding_main.cpp")]
    if against_reference:
        inc += ["-I", os.path.join(O.REF_SRC, "include")]
        srcs.append(os.path.join(O.REF_SRC, "src", "Scene.cpp"))
    else:
        inc += ["-I", TCPP]
        srcs.append(os.path.join(TCPP, "scene_standin.cpp"))
    cmd = (["g++", "-std=c++11", "-O2", "-ffp-contract=off", "-Wall"] + inc + srcs +
           ["-L", lib_dir, "-lminirender_gpu", "-Wl,-rpath," + lib_dir, "-o", exe])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _floats(a) -> str:
    return " ".join(repr(float(x)) for x in np.asarray(a, np.float32).reshape(-1))


def _material(m, tex_index) -> str:
    return f"{_floats(m.diffuse)} {_floats(m.specular)} {_floats(m.emissive)} {float(m.shininess)!r} {tex_index}"


class SceneWriter:
    """Writes the driver's scene description (see binding_main.cpp)."""

    def __init__(self, out_dir: str):
        self.dir = out_dir
        self.lines = []
        self.meshes = {}
        self.textures = {}

    def texture(self, tex) -> int:
        if id(tex) not in self.textures:
            k = len(self.textures)
            # Material::texture holds texels as loadPPM leaves them: b / 255.0f
            t = tex.astype(np.float32) / np.float32(255) if tex.dtype == np.uint8 else tex.astype(np.float32)
            path = os.path.join(self.dir, f"tex{k}.f32")
            np.ascontiguousarray(t).tofile(path)
            self.lines.append(f"texture {k} {tex.shape[0]} {tex.shape[1]} {path}")
            self.textures[id(tex)] = (k, tex)
        return self.textures[id(tex)][0]

    def mesh(self, m) -> int:
        if id(m) not in self.meshes:
            k = len(self.meshes)
            path = os.path.join(self.dir, f"mesh{k}.bin")
            with open(path, "wb") as f:
                for a, t in ((m.vertices, np.float32), (m.normals, np.float32), (m.texcoords, np.float32),
                             (m.indices, np.int32), (m.normalsI, np.int32), (m.texcoordsI, np.int32)):
                    f.write(np.ascontiguousarray(a, t).tobytes())
            self.lines.append(f"mesh {k} {path} {m.vertices.shape[0]} {m.normals.shape[0]} {m.texcoords.shape[0]} "
                              f"{m.indices.size} {m.normalsI.size} {m.texcoordsI.size}")
            self.meshes[id(m)] = (k, m)
        return self.meshes[id(m)][0]

    def state(self, st):
        f = st.to_c()
        self.lines += [f"size {st.width} {st.height}", f"projection {_floats(list(f.projection))}",
                       f"view {_floats(list(f.view))}", f"light {_floats(list(f.light))} {int(f.light_is_point)}",
                       f"background {_floats(list(f.background))}",
                       f"switches {int(st.lighting)} {int(st.texturing)} {int(st.save_normals)}"]

    def scene(self, sc):
        flat = S.flatten(sc)
        mk = [self.mesh(m) for m in flat.meshes]
        tk = [self.texture(t) for t in flat.textures]
        for i in range(len(flat.nodes)):
            nd = flat.nodes[i]
            mesh = mk[nd.mesh] if nd.mesh >= 0 else -1
            mat = S.Material()
            tex = -1
            if nd.has_material:
                mat = S.Material(diffuse=list(nd.material.diffuse), specular=list(nd.material.specular),
                                 emissive=list(nd.material.emissive), shininess=nd.material.shininess)
                tex = tk[nd.material.texture] if nd.material.texture >= 0 else -1
            self.lines.append(f"node {nd.parent} {mesh} {int(nd.has_material)} {_material(mat, tex)} "
                              f"{_floats(list(nd.transform))}")
        self.lines.append(f"ambient {float(np.float32(getattr(sc, 'ambientLight', 0.1)))!r}")

    def paints(self, paints):
        for p in paints:
            if isinstance(p, tuple):  # state calls between paints
                if p[0] == "view":
                    self.lines.append(f"view {_floats(list(np.asarray(p[1], np.float32).reshape(16)))}")
                elif p[0] in ("lighting", "texturing"):
                    self.lines.append(f"{p[0]} {int(bool(p[1]))}")
                elif p[0] == "light":
                    self.lines.append(f"light {_floats(p[1])} {int(bool(p[2]))}")
                elif p[0] == "background":
                    self.lines.append(f"background {_floats(p[1])}")
                else:
                    raise ValueError(p[0])
                continue
            tex = self.texture(p.material.texture) if p.material.texture is not None else -1
            if p.flags & abi.MR_RS_MODELVIEW:
                world = 0 if p.flags & abi.MR_RS_NO_CLIP else 1
                self.lines.append(f"material {_material(p.material, tex)}")
                m = p.mesh
                for t in range(m.indices.size // 3):
                    corners = [f"{_floats(m.vertices[3 * t + c])} {_floats(m.normals[3 * t + c])} "
                               f"{_floats(m.texcoords[3 * t + c])}" for c in range(3)]
                    self.lines.append(f"triangle {world} " + " ".join(corners))
            else:
                k = self.mesh(p.mesh)
                self.lines.append(f"paintmesh {k} 1 {_material(p.material, tex)} {_floats(p.transform)}")

    def write(self) -> str:
        path = os.path.join(self.dir, "scene.txt")
        with open(path, "w") as f:
            f.write("\n".join(self.lines) + "\n")
        return path


def run_driver(exe: str, scene_txt: str) -> subprocess.CompletedProcess:
    return subprocess.run([exe, scene_txt], capture_output=True, text=True, timeout=600)


def read_outputs(prefix: str, st) -> dict:
    H, W_ = st.height, st.width
    out = {"image": np.fromfile(prefix + ".image", np.float32).reshape(H, W_, 3),
           "depth": np.fromfile(prefix + ".depth", np.float32).reshape(H, W_),
           "rgb8": np.fromfile(prefix + ".rgb8", np.uint8).reshape(H, W_, 3),
           "ids": np.fromfile(prefix + ".ids", np.uint32).reshape(H, W_),
           "range": np.fromfile(prefix + ".range", np.float32).reshape(H, W_, 3)}
    if os.path.exists(prefix + ".normals"):
        out["normals"] = np.fromfile(prefix + ".normals", np.float32).reshape(H, W_, 3)
    return out


# ---------------------------------------------------------------- CPU
@pytest.mark.parametrize("against_reference", [False, True], ids=["standin", "reference"])
def test_binding_builds_and_refuses_without_device(product_lib, tmp_path, against_reference):
    """Without a usable GPU the binding throws GpuError(MR_E_NO_DEVICE)
    from its constructor: no CPU path stands in for the device."""
    from conftest import gpu_available
    if against_reference and not os.path.isdir(os.path.join(O.REF_SRC, "src")):
        pytest.skip("reference sources not present on this machine")
    exe = build_driver(str(tmp_path), against_reference)
    if gpu_available():
        pytest.skip("a GPU is present")
    w = SceneWriter(str(tmp_path))
    st, sc = W.config1(32, 24)
    w.state(st)
    w.scene(sc)
    w.lines += ["render", f"out {tmp_path}/o"]
    r = run_driver(exe, w.write())
    assert r.returncode == 3 and r.stdout.startswith(f"GpuError {abi.MR_E_NO_DEVICE}"), r.stdout + r.stderr


# ---------------------------------------------------------------- GPU
def _cases():
    yield "config1_640x480", W.config1(), None
    yield "config2_textured_320x240", W.config2(level=5, width=320, height=240, tex_size=64), None
    import edge_scenes as E
    for seed in (3, 8, 21):
        st, sc = E.random_scene(seed)
        yield f"random_{seed}", st, sc
    st, sc = W.config1(160, 120)
    _, paints = E.paint_sequence(160, 120)
    yield "render_then_paints", st, (sc, paints, paints)
    st, calls, paints = E.view_change_paints(160, 120)
    yield "paints_after_view_change", st, (W.config1(160, 120)[1], calls, paints)
    st, calls, paints = E.state_change_paints(160, 120)
    yield "paints_after_state_changes", st, (W.config1(160, 120)[1], calls, paints)


def _fix(case):
    name, st, sc = case
    if sc is None:
        st, sc = st
    return name, st, sc


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(_cases()), ids=lambda c: c[0])
def test_binding_matches_oracle(product_lib, tmp_path, case):
    name, st, sc = _fix(case)
    exe = build_driver(str(tmp_path))
    w = SceneWriter(str(tmp_path))
    w.state(st)
    if isinstance(sc, tuple):
        base, calls, paints = sc
        w.scene(base)
        w.lines.append("render")
        w.paints(calls)
        ref = O.render_paints(st, paints, base_scene=base)
    else:
        w.scene(sc)
        w.lines.append("render")
        ref = O.render(st, sc, normals=st.save_normals)
    w.lines.append(f"out {tmp_path}/o")
    r = run_driver(exe, w.write())
    assert r.returncode == 0, r.stdout + r.stderr
    got = read_outputs(f"{tmp_path}/o", st)
    stats = compare(got, ref, f"cpp_binding_{name}")
    assert_parity(stats)
    assert np.array_equal(got["range"].view(np.uint32), O.range_image(st, ref["depth"]).view(np.uint32))
    if st.save_normals and "normals" in ref:
        assert np.abs(got["normals"] - ref["normals"]).max() <= 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["textured.obj", "scene.x3d"])
def test_binding_loaded_models(product_lib, tmp_path, name):
    """Models read by the library's loaders render through the binding as
    the oracle renders them."""
    import loader_files
    from minirender_gb300 import loaders
    from minirender_gb300 import projection as pj
    from minirender_gb300.frame import FrameState
    from minirender_gb300.scene import Scene
    loader_files.write_all(str(tmp_path))
    sc = Scene()
    sc.add(loaders.load_mesh(str(tmp_path / name)))
    st = FrameState(width=160, height=120,
                    projection=pj.projection_frustum(pj.deg2rad(50), np.float32(160) / np.float32(120), 0.5, 100),
                    view=pj.translate(0, 0, -6), light=np.array([0.3, 0.5, 1.0], np.float32),
                    ambient=sc.ambientLight)
    exe = build_driver(str(tmp_path))
    w = SceneWriter(str(tmp_path))
    w.state(st)
    w.scene(sc)
    w.lines += ["render", f"out {tmp_path}/o"]
    r = run_driver(exe, w.write())
    assert r.returncode == 0, r.stdout + r.stderr
    got = read_outputs(f"{tmp_path}/o", st)
    ref = O.render(st, sc)
    stats = compare(got, ref, f"cpp_binding_{name}")
    assert_parity(stats)
    assert stats["covered"] > 100


@pytest.mark.gpu
def test_binding_notices_mesh_edits(product_lib, tmp_path):
    """The binding's mesh cache: a mesh scaled in place and announced with
    meshChanged(), then a mesh whose arrays grew (reallocated, longer), are
    each sent again -- every frame equals the oracle's render of the edited
    scene, and each edit changes the picture."""
    from minirender_gb300.scene import Scene, TriMesh
    st, sc0 = W.config1(160, 120)
    m0 = sc0.children[0]
    v0, n0, i0, ni0 = m0.vertices.copy(), m0.normals.copy(), m0.indices.copy(), m0.normalsI.copy()

    def scene_of(v, n, i, ni):
        sc = Scene()
        sc.add(TriMesh(v, n, i, normalsI=ni, material=m0.material))
        return sc

    exe = build_driver(str(tmp_path))
    w = SceneWriter(str(tmp_path))
    w.state(st)
    w.scene(scene_of(v0, n0, i0, ni0))
    # the triangle facing the camera most directly (largest centroid z)
    t = int(np.argmax(v0[i0.reshape(-1, 3)].mean(axis=1)[:, 2]))
    w.lines += ["render", f"out {tmp_path}/a", "scale 1 0.75", "render", f"out {tmp_path}/b",
                f"grow 1 {t}", "render", f"out {tmp_path}/c"]
    r = run_driver(exe, w.write())
    assert r.returncode == 0, r.stdout + r.stderr
    # the same edits on the Python side, in float32 as the driver makes them
    v1 = v0 * np.float32(0.75)
    corner = v1[i0[3 * t:3 * t + 3]].copy()
    corner[:, 2] = corner[:, 2] + np.float32(0.5)
    nv, nn = v1.shape[0], n0.shape[0]
    v2 = np.concatenate([v1, corner])
    n2 = np.concatenate([n0, n0[ni0[3 * t:3 * t + 3]]])
    i2 = np.concatenate([i0, np.arange(nv, nv + 3, dtype=np.int32)])
    ni2 = np.concatenate([ni0, np.arange(nn, nn + 3, dtype=np.int32)])
    previous = None
    for tag, sc in (("a", scene_of(v0, n0, i0, ni0)), ("b", scene_of(v1, n0, i0, ni0)),
                    ("c", scene_of(v2, n2, i2, ni2))):
        got = read_outputs(f"{tmp_path}/{tag}", st)
        stats = compare(got, O.render(st, sc), f"cpp_binding_edit_{tag}")
        assert_parity(stats)
        if previous is not None:
            assert not np.array_equal(got["ids"], previous), f"frame {tag} did not change"
        previous = got["ids"]


@pytest.mark.gpu
def test_binding_frees_meshes_the_frame_drops(product_lib, tmp_path):
    """A node detached from the scene: the next frame no longer draws its
    mesh (the binding frees it); attached again, the mesh is sent again and
    drawn -- every frame equals the oracle's render of the scene as it is."""
    import edge_scenes as E
    from minirender_gb300.scene import Scene
    st, sc1 = W.config1(160, 120)
    sphere = sc1.children[0]
    cube = E._tri_mesh([[-1.2, -1.2, 0.3], [-0.2, -1.2, 0.3], [-0.2, -0.2, 0.3], [-1.2, -0.2, 0.3]],
                       [0, 1, 2, 0, 2, 3], material=sphere.material)
    full = Scene()
    full.add(sphere)
    full.add(cube)
    alone = Scene()
    alone.add(sphere)
    exe = build_driver(str(tmp_path))
    w = SceneWriter(str(tmp_path))
    w.state(st)
    w.scene(full)  # node 0 the scene, 1 the sphere, 2 the quad
    w.lines += ["render", f"out {tmp_path}/a", "detach 2", "render", f"out {tmp_path}/b",
                "attach 2", "render", f"out {tmp_path}/c"]
    r = run_driver(exe, w.write())
    assert r.returncode == 0, r.stdout + r.stderr
    frames = {}
    for tag, sc in (("a", full), ("b", alone), ("c", full)):
        got = read_outputs(f"{tmp_path}/{tag}", st)
        assert_parity(compare(got, O.render(st, sc), f"cpp_binding_detach_{tag}"))
        frames[tag] = got["ids"]
    assert not np.array_equal(frames["a"], frames["b"])
    assert np.array_equal(frames["a"], frames["c"])
