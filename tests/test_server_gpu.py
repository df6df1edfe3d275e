"""Render server (mr_server_*): continuous batching keeps every result equal
to the oracle's render of that request alone, whatever it was batched with;
admission honours the device-memory budget."""
import threading

import numpy as np
import pytest

from minirender_gb300 import abi, capi
from minirender_gb300 import projection as pj
from minirender_gb300 import workloads as W
from oracle import oracle as O
from minirender_gb300.scene import Scene

pytestmark = pytest.mark.gpu


def _pool():
    """(state, mesh) requests of the serving workload: triangle soups of
    various sizes and resolutions plus a textured icosphere."""
    out = []
    for k, (n, w, h) in enumerate([(2000, 160, 120), (20000, 320, 240), (60000, 640, 360), (5000, 128, 128),
                                   (120000, 960, 540)]):
        st, sc = W.config3(n_tris=n, width=w, height=h, seed=40 + k)
        out.append((st, sc.children[0]))
    st, sc = W.config2(level=5, width=400, height=300, tex_size=64)
    out.append((st, sc.children[0]))
    return out


def _oracle(st, mesh):
    sc = Scene()
    sc.add(mesh)
    return O.render(st, sc)


def _buffers(st):
    return {"rgb8": np.zeros((st.height, st.width, 3), np.uint8),
            "depth": np.zeros((st.height, st.width), np.float32),
            "ids": np.zeros((st.height, st.width), np.uint32)}


def _same(a, b):
    return (np.array_equal(a["ids"], b["ids"]) and
            np.array_equal(a["depth"].view(np.uint32), b["depth"].view(np.uint32)) and
            np.abs(a["rgb8"].astype(int) - b["rgb8"].astype(int)).max() <= 1)


@pytest.fixture(scope="module")
def ctx(product_lib):
    c = capi.Context(0)
    yield c
    c.close()


def test_server_matches_oracle_alone_and_in_mix(ctx):
    from minirender_gb300.server import RenderServer
    pool = _pool()
    refs = [_oracle(st, m) for st, m in pool]
    srv = RenderServer(ctx, budget_bytes=8 << 30, slots=2, max_batch=8)
    try:
        # alone: one request at a time
        alone = []
        for i, (st, m) in enumerate(pool):
            out = _buffers(st)
            t = srv.submit(st, m, mesh_key=100 + i, texture_key=900 + i, out=out)
            info = srv.wait(t)
            assert info.status == 0 and info.batch_size == 1
            assert _same(out, refs[i]), f"request {i} alone differs from the oracle"
            alone.append(out)
        # in a mix: every request submitted 4 times from 3 threads, resident
        # meshes re-rendered, batches formed while others run
        results = {}
        lock = threading.Lock()

        def client(tid):
            for rep in range(4):
                for i, (st, m) in enumerate(pool):
                    out = _buffers(st)
                    t = srv.submit(st, m, mesh_key=100 + i, texture_key=900 + i, out=out)
                    with lock:
                        results[t] = (i, out)

        th = [threading.Thread(target=client, args=(k,)) for k in range(3)]
        for x in th:
            x.start()
        for x in th:
            x.join()
        sizes = []
        for t, (i, out) in results.items():
            info = srv.wait(t)
            sizes.append(info.batch_size)
            assert info.status == 0
            assert _same(out, alone[i]), f"request {i} differs between alone and in the mix"
        assert max(sizes) > 1, "no request was batched with another"
        st_ = srv.stats()
        assert st_["completed"] >= len(results) and st_["p99_us"] >= st_["p50_us"] > 0
    finally:
        srv.close()


def test_server_budget_admission_and_eviction(ctx):
    from minirender_gb300.server import RenderServer
    pool = _pool()
    srv = RenderServer(ctx, budget_bytes=64 << 20, slots=2, max_batch=4)
    try:
        st, sc = W.config3(n_tris=2_000_000, width=640, height=480, seed=9)
        with pytest.raises(capi.MRError) as e:
            srv.submit(st, sc.children[0], mesh_key=1)
        assert e.value.code == abi.MR_E_BUDGET
        # many distinct meshes through a small budget: older ones get evicted,
        # every result still matches the oracle
        tickets = []
        for rep in range(3):
            for i, (st, m) in enumerate(pool):
                out = _buffers(st)
                tickets.append((i, out, srv.submit(st, m, mesh_key=1000 * rep + i, texture_key=1000 * rep + i + 500,
                                                   out=out)))
        refs = [_oracle(st, m) for st, m in pool]
        for i, out, t in tickets:
            assert srv.wait(t).status == 0
            assert _same(out, refs[i])
        assert srv.stats()["committed_bytes"] <= 64 << 20
    finally:
        srv.close()


def test_server_other_tunings_same_result(ctx):
    """Every request equals the oracle whatever the server's batch tuning:
    all triangles binned (small_max 0), wide tiles, bigger blocks."""
    from minirender_gb300.server import RenderServer
    pool = _pool()[:4]
    refs = [_oracle(st, m) for st, m in pool]
    for opts in (dict(small_max=0), dict(tile=64, tile_h=16, threads=128, chunk=128, small_max=256)):
        srv = RenderServer(ctx, budget_bytes=8 << 30, slots=2, max_batch=8, **opts)
        try:
            tickets = []
            for rep in range(2):
                for i, (st, m) in enumerate(pool):
                    out = _buffers(st)
                    tickets.append((i, out, srv.submit(st, m, mesh_key=300 + i, texture_key=700 + i, out=out)))
            for i, out, t in tickets:
                assert srv.wait(t).status == 0
                assert _same(out, refs[i]), f"request {i} differs with {opts}"
        finally:
            srv.close()


def test_server_empty_mesh_request(ctx):
    """A request whose mesh has no triangles completes with the background."""
    from minirender_gb300.server import RenderServer
    from minirender_gb300.scene import TriMesh
    st, _ = W.config1(64, 48)
    m = TriMesh(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), np.zeros(0, np.int32))
    srv = RenderServer(ctx, budget_bytes=1 << 30, slots=1, max_batch=4)
    try:
        out = _buffers(st)
        t = srv.submit(st, m, mesh_key=42, out=out)
        assert srv.wait(t).status == 0
        ref = _oracle(st, m)
        assert _same(out, ref)
    finally:
        srv.close()


def test_server_rejects_bad_mesh_descriptors(ctx):
    """Descriptors that mr_mesh_upload refuses (negative counts, a null array
    with a non-zero count, normalsI shorter than indices) are refused at
    submit with MR_E_INVALID, before any queueing; a good request after them
    completes."""
    import ctypes as C
    from minirender_gb300.server import RenderServer
    st, sc = W.config1(64, 48)
    m = sc.children[0]
    srv = RenderServer(ctx, budget_bytes=1 << 30, slots=1, max_batch=4)
    try:
        good = m.desc()
        bad = []
        for field, value in (("n_vertices", -3), ("vertices", None), ("n_normalsI", 3)):
            d = m.desc()
            setattr(d, field, value)
            bad.append(d)
        for d in bad:
            q = abi.mr_request()
            q.frame = st.to_c()
            q.mesh_key = 7
            q.mesh = d
            q.transform[:] = [float(x) for x in np.eye(4, dtype=np.float32).reshape(16)]
            ticket = C.c_uint64(0)
            assert capi.lib().mr_server_submit(srv.h, C.byref(q), C.byref(ticket)) == abi.MR_E_INVALID
        assert good.n_vertices > 0
        out = _buffers(st)
        t = srv.submit(st, m, mesh_key=8, out=out)
        assert srv.wait(t).status == 0
        assert _same(out, _oracle(st, m))
    finally:
        srv.close()


def _random_requests(n=48):
    """First mesh of each seeded random scene (soup or indexed, clipped, both
    projections, odd frame sizes), with its node transform and an RGB8
    texture or none (requests carry RGB8 textures only)."""
    import dataclasses

    import edge_scenes as E
    from minirender_gb300.scene import Material, TriMesh
    out = []
    for seed in range(n):
        st, sc = E.random_scene(seed)
        st = dataclasses.replace(st, save_normals=False)
        m = sc.children[0]
        mat = m.material
        if mat is not None and mat.texture is not None and mat.texture.dtype != np.uint8:
            mat = Material(mat.diffuse, mat.specular, mat.emissive, mat.shininess)
        alone = TriMesh(m.vertices, m.normals, m.indices, normalsI=m.normalsI,
                        texcoords=m.texcoords if m.texcoords.size else None,
                        texcoordsI=m.texcoordsI if m.texcoordsI.size else None, material=mat,
                        transform=m.transform)
        out.append((st, alone))
    return out


def test_server_random_scenes(ctx):
    """Seeded random requests submitted at once from two threads: each
    result equals the oracle's render of that request alone."""
    from minirender_gb300.server import RenderServer
    reqs = _random_requests()
    refs = [_oracle(st, m) for st, m in reqs]
    srv = RenderServer(ctx, budget_bytes=2 << 30, slots=3, max_batch=16)
    try:
        results = {}
        lock = threading.Lock()

        def client(part):
            for i in range(part, len(reqs), 2):
                st, m = reqs[i]
                out = _buffers(st)
                t = srv.submit(st, m, mesh_key=5000 + i, transform=m.transform, texture_key=7000 + i, out=out)
                with lock:
                    results[t] = (i, out)

        th = [threading.Thread(target=client, args=(k,)) for k in range(2)]
        for x in th:
            x.start()
        for x in th:
            x.join()
        for t, (i, out) in results.items():
            assert srv.wait(t).status == 0
            assert _same(out, refs[i]), f"random request {i} differs from the oracle"
        assert len(results) == len(reqs)
    finally:
        srv.close()
