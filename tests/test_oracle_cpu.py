"""CPU tests of the oracle: the C restatement against the reference's own
sources (compiled against the ASL stand-in) where they are present, and
against the committed golden fixtures everywhere."""
import glob
import os

import numpy as np

from minirender_gb300 import abi
import pytest

import edge_scenes as E
from minirender_gb300 import projection as pj
from minirender_gb300 import workloads as W
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32))


def _vs_ref(st, sc, normals=False):
    o = O.render(st, sc, normals=normals)
    r = O.ref_render(st, sc, normals=normals)
    assert _bits_equal(o["image"], r["image"]), "image differs from the reference build"
    assert _bits_equal(o["depth"], r["depth"]), "depth differs from the reference build"
    if normals:
        assert _bits_equal(o["normals"], r["normals"])
    return o


def test_config1_vs_reference(oracle_lib, ref_lib):
    st, sc = W.config1()
    o = _vs_ref(st, sc)
    assert (o["ids"] != 0xFFFFFFFF).sum() > 50_000


def test_config2_reduced_vs_reference(oracle_lib, ref_lib):
    st, sc = W.config2(level=6, width=480, height=270, tex_size=256)
    o = _vs_ref(st, sc)
    assert ((o["ids"] & 1) == 1).sum() > 0  # second half of a clipped quad wins pixels


def test_config3_reduced_vs_reference(oracle_lib, ref_lib):
    st, sc = W.config3(n_tris=100_000, width=640, height=360)
    _vs_ref(st, sc)


@pytest.mark.parametrize("seed", [0, 5])
def test_config4_vs_reference(oracle_lib, ref_lib, seed):
    st, sc = W.config4_scene(seed)
    _vs_ref(st, sc)


@pytest.mark.parametrize("seed", range(48))
def test_random_scene_vs_reference(oracle_lib, ref_lib, seed):
    """Seeded random scenes (tests/edge_scenes.random_scene): soups and
    indexed meshes, nested and instanced nodes, clipping, both projections,
    textures of odd sizes, every lighting switch, normals output."""
    st, sc = E.random_scene(seed)
    _vs_ref(st, sc, normals=st.save_normals)


@pytest.mark.parametrize("name", sorted(E.ALL))
def test_edge_vs_reference(oracle_lib, ref_lib, name):
    st, sc = E.ALL[name]()
    _vs_ref(st, sc, normals=st.save_normals)


def _range_cases():
    yield "config1", W.config1(160, 120)
    for seed in range(0, 48, 4):
        yield f"random{seed}", E.random_scene(seed)


@pytest.mark.parametrize("case", list(_range_cases()), ids=lambda c: c[0])
def test_range_image_vs_reference(oracle_lib, ref_lib, case):
    """Renderer::getRangeImage (depth unprojected to view space), perspective
    and orthographic: the restatement equals the reference build's."""
    st, sc = case[1]
    o = O.render(st, sc)
    r = O.ref_render(st, sc, range_xyz=True)
    assert _bits_equal(O.range_image(st, o["depth"]), r["range"])


def test_primitives_vs_reference(ref_lib):
    """The numpy primitive generators produce the reference's topology and
    its positions within one float32 rounding (trig in double, rounded)."""
    cases = [(W.create_cube(1.0), (0, 1.0, 0, 0, 0)), (W.create_sphere(1.0, 32, 64), (2, 1.0, 0, 32, 64)),
             (W.create_cylinder(0.5, 1.2, 17), (1, 0.5, 1.2, 17, 1))]
    for mesh, (kind, a, b, seg, hseg) in cases:
        ref = O.ref_primitive(kind, a, b, seg, hseg)
        assert np.array_equal(mesh.indices, ref["indices"])
        assert np.array_equal(mesh.normalsI, ref["normalsI"])
        for k in ("vertices", "normals", "texcoords"):
            x, y = getattr(mesh, k), ref[k]
            assert x.shape == y.shape
            assert np.allclose(x, y, rtol=0, atol=1e-6), k


def test_projection_builders_vs_reference(ref_lib):
    np.testing.assert_array_equal(pj.projection_ortho(-40, 40, -30, 30, 50, 120),
                                  O.ref_projection(0, [-40, 40, -30, 30, 50, 120]))
    np.testing.assert_array_equal(pj.projection_perspective(-1, 1.5, -0.7, 0.9, 0.3, 50),
                                  O.ref_projection(1, [-1, 1.5, -0.7, 0.9, 0.3, 50]))
    a = pj.projection_frustum(pj.deg2rad(45), np.float32(640) / np.float32(480), 0.1, 100)
    b = O.ref_projection(2, [pj.deg2rad(45), np.float32(640) / np.float32(480), 0.1, 100])
    np.testing.assert_allclose(a, b, rtol=2e-7)


def test_mat4_ops_vs_reference(ref_lib):
    rng = np.random.default_rng(0)
    for _ in range(200):
        a = rng.normal(size=(4, 4)).astype(np.float32)
        b = rng.normal(size=(4, 4)).astype(np.float32)
        assert _bits_equal(O.mat4_mul(a, b), O.ref_mat4_mul(a, b))
        assert _bits_equal(pj.mat_mul(a, b), O.ref_mat4_mul(a, b))


# ---------------------------------------------------------------- golden fixtures
def _load_fixture(path):
    from golden_io import load_case
    return load_case(path)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_matches_golden(oracle_lib, path):
    """Outputs of the reference's own Renderer, recorded by
    tests/golden/make_golden.py, reproduced bit for bit by the oracle."""
    st, sc, expect = _load_fixture(path)
    o = O.render(st, sc, normals=st.save_normals)
    assert _bits_equal(o["image"], expect["image"])
    assert _bits_equal(o["depth"], expect["depth"])
    if "normals" in expect:
        assert _bits_equal(o["normals"], expect["normals"])


def test_golden_fixtures_present():
    assert len(glob.glob(os.path.join(GOLDEN, "*.npz"))) >= 8


def test_paints_match_reference(ref_lib):
    """paintMesh / paintTriangle sequences: the oracle's restatement is bit
    for bit the reference's own Renderer, after render() and after clear()."""
    import edge_scenes as E
    st, paints = E.paint_sequence()
    for clear in (False, True):
        ref = O.ref_paint(st, paints, clear=clear)
        got = O.render_paints(st, paints)
        assert _bits_equal(got["depth"], ref["depth"]), clear
        assert _bits_equal(got["image"], ref["image"]), clear
        assert (got["ids"] != 0xFFFFFFFF).sum() > 1000


def test_paint_after_view_change_matches_reference(ref_lib):
    """paintMesh after setView uses the new view while the light stays where
    render() placed it: the reference's own Renderer equals the frame as one
    paint list whose later paints carry their modelview (MR_RS_MODELVIEW),
    the form the mirrors hand to the library."""
    import edge_scenes as E
    st, calls, paints = E.view_change_paints()
    got = O.render_paints(st, paints)
    for clear in (False, True):
        ref = O.ref_paint(st, calls, clear=clear)
        assert _bits_equal(got["depth"], ref["depth"]), clear
        assert _bits_equal(got["image"], ref["image"]), clear
    # the view change moved what it drew: the same calls without it differ
    flat = O.render_paints(st, [c for c in calls if not isinstance(c, tuple)])
    assert not _bits_equal(flat["depth"], got["depth"])


def test_paint_after_state_changes_matches_reference(ref_lib):
    """setLighting / setTexturing / setLight / setBackground between paints:
    the reference's own Renderer equals the frame as one paint list whose
    paints carry the switches of their call (MR_RS_OWN_STATE), with the
    light where render() placed it and the background of clear()."""
    import edge_scenes as E
    st, calls, paints = E.state_change_paints()
    got = O.render_paints(st, paints)
    for clear in (False, True):
        ref = O.ref_paint(st, calls, clear=clear)
        assert _bits_equal(got["depth"], ref["depth"]), clear
        assert _bits_equal(got["image"], ref["image"]), clear
    # the switches changed what was drawn: the same paints under the frame's differ
    keep = abi.MR_RS_MODELVIEW | abi.MR_RS_NO_CLIP
    plain = O.render_paints(st, [type(p)(p.mesh, p.transform, p.material, p.flags & keep) for p in paints])
    assert not _bits_equal(plain["image"], got["image"])
    assert _bits_equal(plain["depth"], got["depth"])


def test_paints_match_golden():
    """The oracle's paint sequence against the committed digests of the
    reference's own paintMesh / paintTriangle (tests/golden/paints.json)."""
    import hashlib
    import json
    import edge_scenes as E
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "paints.json")) as f:
        want = json.load(f)
    st, paints = E.paint_sequence()
    for clear in (False, True):
        got = O.render_paints(st, paints)
        for k in ("image", "depth"):
            assert hashlib.sha256(got[k].tobytes()).hexdigest() == want[f"clear{int(clear)}"][k], (clear, k)


@pytest.mark.parametrize("seed", range(32))
def test_random_paints_vs_reference(ref_lib, seed):
    """Seeded random paintMesh / paintTriangle sequences
    (tests/edge_scenes.random_paints): the restatement equals the reference's
    Renderer after render() and after clear()."""
    import edge_scenes as E
    st, paints = E.random_paints(seed)
    got = O.render_paints(st, paints)
    for clear in (False, True):
        ref = O.ref_paint(st, paints, clear=clear)
        assert _bits_equal(got["depth"], ref["depth"]), clear
        assert _bits_equal(got["image"], ref["image"]), clear


@pytest.mark.parametrize("name", ["view_change", "state_changes"])
def test_state_paints_match_golden(name):
    """Paints around setView / setLighting / setTexturing / setLight /
    setBackground: the oracle's one-list form against the committed digests
    of the reference's Renderer (tests/golden/paints.json)."""
    import hashlib
    import json
    import edge_scenes as E
    with open(os.path.join(GOLDEN, "paints.json")) as f:
        want = json.load(f)[name]
    make = E.view_change_paints if name == "view_change" else E.state_change_paints
    st, _, paints = make()
    got = O.render_paints(st, paints)
    for k in ("image", "depth"):
        assert hashlib.sha256(got[k].tobytes()).hexdigest() == want[k], k


@pytest.mark.parametrize("seed", range(8))
def test_random_paints_match_golden(seed):
    """Random paint sequences against the committed digests of the
    reference's Renderer (tests/golden/paints.json; no reference build needed)."""
    import hashlib
    import json
    import edge_scenes as E
    with open(os.path.join(GOLDEN, "paints.json")) as f:
        want = json.load(f)[f"random/{seed}"]
    got = O.render_paints(*E.random_paints(seed))
    for k in ("image", "depth"):
        assert hashlib.sha256(got[k].tobytes()).hexdigest() == want[k], k
