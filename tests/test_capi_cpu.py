"""CPU tests of the C-ABI library: it loads, exports every entry point the
header declares, its struct layouts match the ctypes mirror, and its host
helpers (matrix arithmetic, projections, collectShapes) agree bit for bit
with the oracle.  No device work is issued."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from minirender_gb300 import abi, capi
from minirender_gb300 import projection as pj
from minirender_gb300 import scene as S
from minirender_gb300 import workloads as W
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", "minirender_gpu.h")]


def declared():
    names = []
    for h in HEADERS:
        txt = open(h).read()
        names += re.findall(r"MR_API\s+[\w\s\*]+?\b(mr_\w+)\s*\(", txt)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared()
    assert "mr_render" in names and "mr_create" in names and len(names) >= 25


def test_library_exports_every_declared_symbol(product_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", capi.LIB], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\sT\s+(mr_\w+)", out))
    missing = [n for n in declared() if n not in exported]
    assert not missing, missing
    for n in declared():
        assert hasattr(product_lib, n)
    assert set(capi.declared_symbols()) <= set(declared())


def test_struct_layouts_match_ctypes(tmp_path):
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include "minirender_gpu.h"\n'
                   'int main(){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(mr_material), '
                   'sizeof(mr_mesh_desc), sizeof(mr_renderable), sizeof(mr_node), sizeof(mr_frame), '
                   'sizeof(mr_outputs), sizeof(mr_stats), sizeof(mr_batch_scene), sizeof(mr_server_opts), '
                   'sizeof(mr_request), sizeof(mr_request_info), sizeof(mr_server_stats));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    want = [C.sizeof(t) for t in (abi.mr_material, abi.mr_mesh_desc, abi.mr_renderable, abi.mr_node,
                                  abi.mr_frame, abi.mr_outputs, abi.mr_stats, abi.mr_batch_scene,
                                  abi.mr_server_opts, abi.mr_request, abi.mr_request_info,
                                  abi.mr_server_stats)]
    assert got == want


@pytest.mark.parametrize("lang", ["c99", "c++11"])
def test_header_compiles_strictly(tmp_path, lang):
    """A plain C or C++ consumer (an FFI stub, a cgo preamble) includes the
    header with every warning as an error."""
    ext, cc = (".c", "gcc") if lang == "c99" else (".cpp", "g++")
    src = tmp_path / ("h" + ext)
    src.write_text('#include "minirender_gpu.h"\nint main(void) { return MR_ABI_VERSION > 0 ? 0 : 1; }\n')
    subprocess.run([cc, f"-std={lang}", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(tmp_path / "h")], check=True)


def test_abi_version_and_status(product_lib):
    assert product_lib.mr_abi_version() == 2
    assert product_lib.mr_status_string(abi.MR_E_BAD_INDEX) == b"mesh index out of range"


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_mat4_helpers_match_oracle(product_lib, oracle_lib):
    rng = np.random.default_rng(1)
    for _ in range(300):
        a = rng.normal(size=(4, 4)).astype(np.float32)
        b = rng.normal(size=(4, 4)).astype(np.float32)
        assert np.array_equal(_bits(capi.mat4_mul(a, b)), _bits(O.mat4_mul(a, b)))
        assert np.array_equal(_bits(capi.mat4_inverse(a)), _bits(O.mat4_inverse(a)))


def test_projection_helpers(product_lib):
    np.testing.assert_array_equal(capi.projection("ortho", -40, 40, -30, 30, 50, 120),
                                  pj.projection_ortho(-40, 40, -30, 30, 50, 120))
    np.testing.assert_array_equal(capi.projection("perspective", -1, 1.5, -0.7, 0.9, 0.3, 50),
                                  pj.projection_perspective(-1, 1.5, -0.7, 0.9, 0.3, 50))
    np.testing.assert_allclose(capi.projection("frustum", 0.8, 1.5, 0.1, 100),
                               pj.projection_frustum(0.8, 1.5, 0.1, 100), rtol=2e-7)


def test_projection_helpers_vs_reference(product_lib, ref_lib):
    """mr_projection_* against the reference's own projection builders."""
    fov = pj.deg2rad(35)
    asp = np.float32(1920) / np.float32(1080)
    np.testing.assert_array_equal(capi.projection("frustum", fov, asp, 10, 7000),
                                  O.ref_projection(2, [fov, asp, 10, 7000]))
    np.testing.assert_array_equal(capi.projection("frustum_h", fov, asp, 10, 7000),
                                  O.ref_projection(3, [fov, asp, 10, 7000]))
    np.testing.assert_array_equal(capi.projection("ortho_fov", 20, asp, 1, 70),
                                  O.ref_projection(4, [20, asp, 1, 70]))


def test_collect_shapes_matches_oracle(product_lib, oracle_lib):
    for seed in range(4):
        st, sc = W.config4_scene(seed)
        flat = S.flatten(sc)
        a, na = capi.collect_shapes(flat.nodes)
        b, nb = O.collect_shapes(flat)
        assert na == nb == 64
        assert C.string_at(C.addressof(a), C.sizeof(abi.mr_renderable) * na) == \
            C.string_at(C.addressof(b), C.sizeof(abi.mr_renderable) * nb)


def test_collect_shapes_random_trees_match_oracle(product_lib, oracle_lib):
    """Nested groups, meshes under meshes and instanced meshes of the seeded
    random scenes: the library's collectShapes equals the oracle's bytes."""
    import edge_scenes as E
    for seed in range(48):
        st, sc = E.random_scene(seed)
        flat = S.flatten(sc)
        a, na = capi.collect_shapes(flat.nodes)
        b, nb = O.collect_shapes(flat)
        assert na == nb >= 1
        assert C.string_at(C.addressof(a), C.sizeof(abi.mr_renderable) * na) == \
            C.string_at(C.addressof(b), C.sizeof(abi.mr_renderable) * nb), seed


def test_collect_shapes_rejects_bad_trees(product_lib):
    nodes = (abi.mr_node * 2)()
    nodes[0].parent = -1
    nodes[0].mesh = -1
    nodes[1].parent = 5
    out = (abi.mr_renderable * 2)()
    n = C.c_int32()
    assert product_lib.mr_collect_shapes(C.addressof(nodes), 2, C.addressof(out), 2, C.byref(n)) == abi.MR_E_INVALID


def test_no_device_is_reported_not_faked(product_lib):
    """Without a GPU the library refuses to create a context (no CPU path)."""
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert product_lib.mr_create(0, C.byref(h)) == abi.MR_E_NO_DEVICE
    with pytest.raises(capi.MRError):
        capi.Context(0)


def _noalloc_call(lib, desc, width=64, height=48):
    st, _ = W.config1(width, height)
    frame = st.to_c()
    mat = abi.mr_material()
    xf = (C.c_float * 16)(*np.eye(4, dtype=np.float32).reshape(16))
    return lib.mr_render_noalloc(C.byref(frame), C.byref(desc), C.addressof(xf), C.byref(mat),
                                 None, 0, 0, 0, None, None, None, None)


@pytest.mark.parametrize("field", ["vertices", "normals", "indices", "normalsI", "texcoords", "texcoordsI"])
def test_noalloc_rejects_null_arrays_before_device_work(product_lib, field):
    """mr_render_noalloc takes device pointers it cannot inspect: an array
    given as NULL with a non-zero count is refused (MR_E_INVALID) before any
    device work, as mr_mesh_upload refuses it, instead of reaching a kernel
    as address 0.  The call returns before touching a device, so this runs
    without a GPU."""
    fake = 1 << 40  # never dereferenced: the checks run first
    d = abi.mr_mesh_desc(fake, 3, fake, 3, fake, 3, fake, 3, fake, 3, fake, 3)
    setattr(d, field, None)
    assert _noalloc_call(product_lib, d) == abi.MR_E_INVALID


@pytest.mark.parametrize("bad", [{"n_normalsI": -3}, {"n_texcoordsI": -3}, {"n_vertices": -1},
                                 {"n_indices": 4, "n_normalsI": 4, "n_texcoordsI": 4},
                                 {"n_normalsI": 0}, {"n_texcoordsI": 1}])
def test_noalloc_rejects_bad_counts_before_device_work(product_lib, bad):
    fake = 1 << 40
    d = abi.mr_mesh_desc(fake, 3, fake, 3, fake, 3, fake, 3, fake, 3, fake, 3)
    for k, v in bad.items():
        setattr(d, k, v)
    assert _noalloc_call(product_lib, d) == abi.MR_E_INVALID


def test_noalloc_limits_checked_before_device_work(product_lib):
    """Frames larger than the fixed scratch give MR_E_NOALLOC_LIMIT (an empty
    mesh: nothing could be dereferenced even if the check were missing)."""
    d = abi.mr_mesh_desc()
    for w, h in ((abi.MR_NOALLOC_MAX_SIDE + 1, 16), (2048, 2048)):
        assert _noalloc_call(product_lib, d, w, h) == abi.MR_E_NOALLOC_LIMIT


def test_header_constants_match_abi():
    """Every integer #define of include/minirender_gpu.h that the Python ABI
    mirrors has the same value there; the renderable flags are all mirrored."""
    import re
    from minirender_gb300 import abi
    with open(os.path.join(ROOT, "include", "minirender_gpu.h")) as f:
        txt = f.read()
    # plain literals only (a value written as an expression is skipped)
    defs = dict(re.findall(r"^#define\s+(MR_\w+)\s+\(?(-?(?:0x[0-9a-fA-F]+|\d+))\)?[ \t]*(?:/\*.*)?$", txt, re.M))
    assert {k for k in defs if k.startswith("MR_RS_")} <= set(dir(abi))
    checked = 0
    for name, value in defs.items():
        if hasattr(abi, name):
            assert getattr(abi, name) == int(value, 0), name
            checked += 1
    assert checked >= 10
