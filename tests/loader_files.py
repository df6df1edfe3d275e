"""Seeded sample files for the loader tests: ASCII and binary STL, OBJ with
material libraries, polygons and every face-index form, OBJ without normals,
X3D with transforms, DEF/USE, both face-set kinds and an Inline, and PPM
images with header comments.  write_all(dir) writes them and returns the
list of model paths (relative names)."""
import os
import struct

import numpy as np


def _ppm(path, rgb, comment=False):
    rows, cols = rgb.shape[:2]
    head = b"P6\n" + (b"# made by the loader tests\n" if comment else b"") + f"{cols} {rows}\n255\n".encode()
    with open(path, "wb") as f:
        f.write(head + np.ascontiguousarray(rgb, np.uint8).tobytes())


def _fmt(x):
    return repr(float(np.float32(x)))


def write_all(d):
    rng = np.random.default_rng(11)
    names = []

    # --- ASCII STL: mixed spacing, CRLF lines, a facet with 4 vertices (dropped)
    lines = ["solid sample part"]
    for k in range(40):
        n = rng.normal(size=3)
        v = rng.uniform(-2, 2, (3, 3))
        lines.append(f"  facet normal {_fmt(n[0])} {_fmt(n[1])}  {_fmt(n[2])}")
        lines.append("    outer loop")
        for p in v:
            lines.append(f"\tvertex {_fmt(p[0])} {_fmt(p[1])} {_fmt(p[2])}")
        if k == 7:
            lines.append(f"    vertex 0.5 0.25 {_fmt(v[0, 2])}")
        lines.append("    endloop")
        lines.append("  endfacet")
    lines.append("endsolid sample part")
    with open(os.path.join(d, "ascii.stl"), "wb") as f:
        f.write("\r\n".join(lines).encode() + b"\r\n")
    names.append("ascii.stl")

    # --- binary STL (header, count, 50-byte facets)
    nf = 300
    with open(os.path.join(d, "binary.stl"), "wb") as f:
        f.write(b"binary sample".ljust(80, b" "))
        f.write(struct.pack("<i", nf))
        for k in range(nf):
            vals = rng.normal(size=12).astype(np.float32)
            f.write(vals.tobytes() + struct.pack("<h", k % 7))
    names.append("binary.stl")

    # --- textures
    _ppm(os.path.join(d, "wood.ppm"), rng.integers(0, 256, (16, 24, 3)), comment=True)
    _ppm(os.path.join(d, "tex.ppm"), rng.integers(0, 256, (8, 8, 3)))

    # --- OBJ with materials, polygons, every face form
    with open(os.path.join(d, "parts.mtl"), "w") as f:
        f.write("Kd 0.5 0.5 0.5\n")  # before any newmtl: the default material
        f.write("newmtl red\nKd 0.9 0.1 0.1\nKs 0.2 0.2 0.2\nKe 0.01 0 0\nNs 0\n")
        f.write("newmtl wood\nKd 0.6 0.4 0.2\nNs 32\nd 0.5\nmap_Kd wood.ppm\n")
        f.write("newmtl missing_tex\nmap_Kd nothere.ppm\n")
    nv = 60
    with open(os.path.join(d, "parts.obj"), "w", newline="") as f:
        f.write("# sample\r\nmtllib parts.mtl\r\n")
        for p in rng.uniform(-1, 1, (nv, 3)):
            f.write(f"v {_fmt(p[0])} {_fmt(p[1])} {_fmt(p[2])}\n")
        for p in rng.normal(size=(nv, 3)):
            f.write(f"vn {_fmt(p[0])} {_fmt(p[1])} {_fmt(p[2])}\n")
        for p in rng.uniform(0, 1, (nv, 2)):
            f.write(f"vt {_fmt(p[0])} {_fmt(p[1])}\n")
        f.write("\n")
        for k in range(30):
            if k % 10 == 0:
                f.write(["usemtl red\n", "usemtl wood\n", "usemtl nosuch\n"][k // 10])
            m = 3 + k % 3  # triangles, quads, pentagons
            ids = rng.choice(nv, m, replace=False) + 1
            form = k % 4
            if form == 0:
                toks = [f"{i}/{i}/{i}" for i in ids]
            elif form == 1:
                toks = [f"{i}//{i}" for i in ids]
            elif form == 2:
                toks = [f"{i}/{i}" for i in ids]
            else:
                toks = [f"{i}" for i in ids]
            f.write("f " + " ".join(toks) + "\n")
        f.write("usemtl red\nf 1/1/1 2/2/2 3/3/3\n")
    names.append("parts.obj")

    # --- a well-formed textured OBJ (every face v/vt/vn): renderable as is
    with open(os.path.join(d, "textured.obj"), "w") as f:
        f.write("mtllib parts.mtl\nusemtl wood\n")
        for p in rng.uniform(-1, 1, (nv, 3)):
            f.write(f"v {_fmt(p[0])} {_fmt(p[1])} {_fmt(p[2])}\n")
        for p in rng.normal(size=(nv, 3)):
            f.write(f"vn {_fmt(p[0])} {_fmt(p[1])} {_fmt(p[2])}\n")
        for p in rng.uniform(0, 2, (nv, 2)):
            f.write(f"vt {_fmt(p[0])} {_fmt(p[1])}\n")
        for k in range(40):
            ids = rng.choice(nv, 3 + k % 3, replace=False) + 1
            f.write("f " + " ".join(f"{i}/{i}/{i}" for i in ids) + "\n")
            if k == 20:
                f.write("usemtl red\n")
    names.append("textured.obj")

    # --- OBJ without normals (face normals generated) and no material library
    with open(os.path.join(d, "plain.obj"), "w") as f:
        for p in rng.uniform(-1, 1, (20, 3)):
            f.write(f"v {_fmt(p[0])} {_fmt(p[1])} {_fmt(p[2])}\n")
        for k in range(15):
            ids = rng.choice(20, 3 + k % 2, replace=False) + 1
            f.write("f " + " ".join(str(i) for i in ids) + "\n")
    names.append("plain.obj")

    # --- X3D: transforms, groups, DEF/USE, face and triangle sets, Inline
    coords = " ".join(_fmt(x) for x in rng.uniform(-1, 1, 3 * 12))
    normals = ",".join(_fmt(x) for x in rng.normal(size=3 * 12))
    uvs = " ".join(_fmt(x) for x in rng.uniform(0, 1, 2 * 12))
    with open(os.path.join(d, "inner.x3d"), "w") as f:
        f.write('<?xml version="1.0"?>\n<X3D><Scene>\n'
                '<Shape><IndexedTriangleSet index="0 1 2 2 3 0"><Coordinate point="0 0 0 1 0 0 1 1 0 0 1 0"/>'
                '</IndexedTriangleSet></Shape>\n</Scene></X3D>\n')
    with open(os.path.join(d, "scene.x3d"), "w") as f:
        f.write('<?xml version="1.0" encoding="UTF-8"?>\n'
                '<!DOCTYPE X3D PUBLIC "ISO//Web3D//DTD X3D 3.2//EN" "x3d-3.2.dtd">\n'
                '<X3D profile="Interchange"><head><meta name="generator" content="tests"/></head>\n<Scene>\n'
                '<!-- a comment -->\n'
                '<Transform translation="1 -2 0.5" rotation="0 1 1 0.7" scale="2 1 0.5">\n'
                ' <Shape><Appearance><Material DEF="M1" diffuseColor="0.2 0.4 0.6" specularColor="1 1 1" '
                'shininess="0.25"/><ImageTexture url="tex.png"/></Appearance>\n'
                f'  <IndexedFaceSet coordIndex="0 1 2 3 -1 4 5 6 -1 7 8 9 10 11 -1" '
                'normalIndex="0 1 2 3 -1 4 5 6 -1 7 8 9 10 11 -1" texCoordIndex="">\n'
                f'   <Coordinate DEF="C1" point="{coords}"/><Normal vector="{normals}"/>'
                f'<TextureCoordinate point="{uvs}"/>\n'
                '  </IndexedFaceSet></Shape>\n'
                ' <Group><Shape><Appearance><Material USE="M1"/></Appearance>'
                '<IndexedFaceSet coordIndex="0 2 4 6 -1 1 3 5"><Coordinate USE="C1"/></IndexedFaceSet></Shape>'
                '</Group>\n'
                '</Transform>\n'
                '<Shape><IndexedTriangleSet index="0 1 2 3 4 5"><Coordinate USE="C1"/></IndexedTriangleSet></Shape>\n'
                '<Shape><Appearance><ImageTexture url=\'"tex.png" "http://example.invalid/tex.png"\'/>'
                '</Appearance></Shape>\n'
                '<Shape/>\n'
                '<Inline url=\'"inner.x3d"\'/>\n'
                '<Unknown/>\n'
                '</Scene></X3D>\n')
    names.append("scene.x3d")
    return names
