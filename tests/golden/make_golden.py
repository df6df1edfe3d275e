#!/usr/bin/env python3
"""Regenerates tests/golden/*.npz: small seeded scenes rendered by the
reference's own Renderer (src/Renderer.cpp, src/Scene.cpp compiled unmodified
against the ASL stand-in by oracle/Makefile).  Needs the reference sources;
run from the repository root:  python tests/golden/make_golden.py
Each fixture stores its inputs, so the check does not depend on the
platform's math library regenerating identical scenes."""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import edge_scenes as E  # noqa: E402
from golden_io import save_case  # noqa: E402
from minirender_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402


def cases():
    yield "config1_128x96", W.config1(128, 96)
    yield "config2_l4_128x72", W.config2(level=4, width=128, height=72, tex_size=32)
    yield "config3_4k_128x72", W.config3(n_tris=4000, width=128, height=72)
    st, sc = W.config4_scene(3, n_prims=10, resolution=(128, 96))
    yield "config4_s3_128x96", (st, sc)
    for name, fn in sorted(E.ALL.items()):
        yield "edge_" + name, fn(128, 96) if name == "big_triangles" else fn()
    for seed in range(4):
        yield f"random_s{seed}", E.random_scene(seed)


def loader_digests():
    """tests/golden/loaders.json: digests of the reference loaders' output
    (src/io.cpp, src/x3d.cpp) for the seeded sample files and the seeded
    random files of tests/loader_files.py, serialised as
    tests/test_loaders_cpu.py does."""
    import json
    import tempfile

    import loader_files
    import test_loaders_cpu as T
    with tempfile.TemporaryDirectory() as d:
        out = {n: T.digest(O.ref_load_mesh(os.path.join(d, n))) for n in loader_files.write_all(d)}
    for key, make in T.RANDOM_FILES:
        with tempfile.TemporaryDirectory() as d:
            out[key] = T.digest(O.ref_load_mesh(os.path.join(d, make(d))))
    with open(os.path.join(HERE, "loaders.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("loaders.json:", ", ".join(sorted(out)))


def paint_digests():
    """tests/golden/paints.json: digests of the reference Renderer's image and
    depth for the paintMesh / paintTriangle sequence of
    tests/edge_scenes.paint_sequence, after render() and after clear(), and
    for the seeded random sequences of tests/edge_scenes.random_paints, and
    for the paints around setView / setLighting / setTexturing / setLight /
    setBackground calls of tests/edge_scenes.view_change_paints and
    state_change_paints."""
    import hashlib
    import json
    st, paints = E.paint_sequence()
    out = {}
    for clear in (False, True):
        r = O.ref_paint(st, paints, clear=clear)
        out[f"clear{int(clear)}"] = {k: hashlib.sha256(r[k].tobytes()).hexdigest() for k in ("image", "depth")}
    for seed in range(8):  # tests/edge_scenes.random_paints, after clear()
        r = O.ref_paint(*E.random_paints(seed), clear=True)
        out[f"random/{seed}"] = {k: hashlib.sha256(r[k].tobytes()).hexdigest() for k in ("image", "depth")}
    for name, make in (("view_change", E.view_change_paints), ("state_changes", E.state_change_paints)):
        st, calls, _ = make()
        r = O.ref_paint(st, calls)
        out[name] = {k: hashlib.sha256(r[k].tobytes()).hexdigest() for k in ("image", "depth")}
    with open(os.path.join(HERE, "paints.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("paints.json:", ", ".join(sorted(out)))


def main():
    if O.ref_lib() is None:
        sys.exit("reference sources not available")
    loader_digests()
    paint_digests()
    for name, (st, sc) in cases():
        r = O.ref_render(st, sc, normals=st.save_normals)
        expect = {"image": r["image"], "depth": r["depth"]}
        if st.save_normals:
            expect["normals"] = r["normals"]
        path = os.path.join(HERE, name + ".npz")
        save_case(path, st, sc, expect)
        print(f"{name}: {os.path.getsize(path) / 1024:.0f} KiB")


if __name__ == "__main__":
    main()
