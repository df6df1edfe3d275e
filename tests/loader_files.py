"""Seeded sample files for the loader tests: ASCII and binary STL, OBJ with
material libraries, polygons and every face-index form, OBJ without normals,
X3D with transforms, DEF/USE, both face-set kinds and an Inline, and PPM
images with header comments.  write_all(dir) writes them and returns the
list of model paths (relative names); random_obj, random_ascii_stl and
random_x3d write one seeded random file each for the loader fuzz tests."""
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


def _num(rng, x):
    """One float in a random textual form (all parse to nearby values)."""
    k = int(rng.integers(5))
    x = float(np.float32(x))
    if k == 0:
        return repr(x)
    if k == 1:
        return f"{x:.4f}"
    if k == 2:
        return f"{x:.6e}"
    if k == 3:
        return f"{x:g}"
    return f"{x:+.9g}"


def _sep(rng):
    return [" ", " ", "  ", "\t", " \t "][int(rng.integers(5))]


def random_obj(d, seed):
    """A seeded random OBJ + MTL pair: random counts of v / vn / vt (some
    files without normals or texcoords), polygons of 3-6 corners in every
    face form (v, v/vt, v//vn, v/vt/vn, and rarely v/vt/ with an empty
    field), usemtl switches among defined, undefined and not-yet-defined
    materials with mtllib at a random place, comments, blank lines, o / g / s
    lines, tabs and runs of spaces, CRLF or LF, numbers in several notations;
    materials with Kd before any newmtl, Ns 0, opacity, present and missing
    textures.  Returns the OBJ's file name."""
    rng = np.random.default_rng(500 + seed)
    stem = f"rand{seed}"
    nl = "\r\n" if rng.random() < 0.3 else "\n"
    rows, cols = int(rng.integers(1, 9)), int(rng.integers(1, 9))
    _ppm(os.path.join(d, stem + ".ppm"), rng.integers(0, 256, (rows, cols, 3)), comment=rng.random() < 0.5)
    nmat = int(rng.integers(0, 5))
    mt = []
    if rng.random() < 0.3:
        mt.append("Kd" + "".join(_sep(rng) + _num(rng, v) for v in rng.uniform(0, 1, 3)))
    for k in range(nmat):
        mt.append(f"newmtl m{k}")
        for key in ("Kd", "Ks", "Ke"):
            if rng.random() < 0.7:
                mt.append(key + "".join(_sep(rng) + _num(rng, v) for v in rng.uniform(0, 1, 3)))
        if rng.random() < 0.6:
            mt.append("Ns" + _sep(rng) + ("0" if rng.random() < 0.25 else _num(rng, rng.uniform(1, 100))))
        if rng.random() < 0.3:
            mt.append("d " + _num(rng, rng.uniform(0, 1)))
        if rng.random() < 0.4:
            mt.append("map_Kd " + (stem + ".ppm" if rng.random() < 0.7 else "absent.ppm"))
        if rng.random() < 0.3:
            mt.append("")
    with open(os.path.join(d, stem + ".mtl"), "w", newline="") as f:
        f.write(nl.join(mt) + nl)

    nv = int(rng.integers(3, 80))
    has_vn, has_vt = rng.random() < 0.7, rng.random() < 0.6
    nn = int(rng.integers(1, 60)) if has_vn else 0
    nt = int(rng.integers(1, 60)) if has_vt else 0
    decl = ["v"] * nv + ["vn"] * nn + ["vt"] * nt
    rng.shuffle(decl)
    lines = ["# random OBJ"]
    for kind in decl:
        if kind == "v":
            vals = rng.uniform(-3, 3, 3)
        elif kind == "vn":
            vals = rng.normal(size=3)
        else:
            vals = rng.uniform(-0.5, 2, 2 + int(rng.random() < 0.2))
        lines.append(kind + "".join(_sep(rng) + _num(rng, v) for v in vals) + (" " if rng.random() < 0.1 else ""))
        if rng.random() < 0.03:
            lines.append("")
    names = [f"m{k}" for k in range(nmat)] + ["undefined"]
    mtllib_at = int(rng.integers(-1, 20))  # face count before the mtllib line (-1: none)
    forms = ["v"] + (["v/vt"] if has_vt else []) + (["v//vn"] if has_vn else []) + \
            (["v/vt/vn"] if has_vt and has_vn else [])
    n_faces = int(rng.integers(1, 60))
    for k in range(n_faces):
        if k == mtllib_at:
            lines.append(f"mtllib {stem}.mtl")
        r = rng.random()
        if r < 0.15:
            lines.append("usemtl " + names[int(rng.integers(len(names)))])
        elif r < 0.18:
            lines.append(["o part", "g group one", "s off", "s 1"][int(rng.integers(4))])
        elif r < 0.2:
            lines.append("# comment f 1 2 3")
        m = int(rng.integers(3, 7))
        ids = rng.choice(nv, min(m, nv), replace=False) + 1
        form = forms[int(rng.integers(len(forms)))]
        toks = []
        for i in ids:
            ti = int(rng.integers(1, nt + 1)) if nt else 0
            ni = int(rng.integers(1, nn + 1)) if nn else 0
            toks.append({"v": f"{i}", "v/vt": f"{i}/{ti}", "v//vn": f"{i}//{ni}",
                         "v/vt/vn": f"{i}/{ti}/{ni}"}[form])
        if has_vt and rng.random() < 0.03:
            toks[0] = f"{ids[0]}/{max(1, nt)}/"
        lines.append("f" + "".join(_sep(rng) + t for t in toks))
    if mtllib_at >= n_faces:
        lines.append(f"mtllib {stem}.mtl")
    with open(os.path.join(d, stem + ".obj"), "w", newline="") as f:
        f.write(nl.join(lines) + (nl if rng.random() < 0.8 else ""))
    return stem + ".obj"


def random_ascii_stl(d, seed):
    """A seeded random ASCII STL: facets of 2-4 vertices (only 3-vertex
    facets become triangles, the others' vertices still count), numbers in
    several notations, tabs and runs of spaces, CRLF or LF, with or without
    a solid name and the closing endsolid.  Returns the file name."""
    rng = np.random.default_rng(700 + seed)
    nl = "\r\n" if rng.random() < 0.4 else "\n"
    lines = ["solid" + (" part_" + str(seed) if rng.random() < 0.7 else "")]
    for k in range(int(rng.integers(1, 60))):
        n = rng.normal(size=3)
        lines.append(_sep(rng) + "facet" + _sep(rng) + "normal" + "".join(_sep(rng) + _num(rng, v) for v in n))
        lines.append(_sep(rng) + "outer loop")
        nvert = 3 if rng.random() < 0.9 else int(rng.choice([2, 4]))
        for p in rng.uniform(-5, 5, (nvert, 3)):
            lines.append(_sep(rng) + "vertex" + "".join(_sep(rng) + _num(rng, v) for v in p))
        lines.append(_sep(rng) + "endloop")
        lines.append(_sep(rng) + "endfacet")
    if rng.random() < 0.8:
        lines.append("endsolid")
    name = f"rand{seed}.stl"
    with open(os.path.join(d, name), "w", newline="") as f:
        f.write(nl.join(lines) + nl)
    return name


def random_x3d(d, seed):
    """A seeded random X3D scene: Transform / Group nodes nested up to three
    deep with random translation, rotation and scale (or none); Shapes with
    or without Appearance, Material (random subset of attributes, DEF and
    USE), ImageTexture (present and missing files); IndexedFaceSet polygons
    of 3-5 corners with and without normalIndex / texCoordIndex and a
    trailing -1, or IndexedTriangleSet; Coordinate DEF / USE; number lists
    separated by spaces, commas or both; both attribute quote styles.
    Returns the file name."""
    rng = np.random.default_rng(900 + seed)
    _ppm(os.path.join(d, f"xrand{seed}.ppm"), rng.integers(0, 256, (int(rng.integers(1, 6)), int(rng.integers(1, 6)), 3)))
    coord_defs = {}  # DEF name -> point count
    mat_defs = []

    def q(v):
        return f"'{v}'" if rng.random() < 0.3 else f'"{v}"'

    def nums(vals, ints=False, spaced=False):
        # Transform fields and index lists are split at whitespace only (a
        # bare comma would merge fields, and the reference reads past the end
        # of a short list); point and vector lists also split at commas
        seps = [" ", ", ", "  "] if spaced or ints else [" ", ", ", ",", "  "]
        sep = seps[int(rng.integers(len(seps)))]
        return sep.join(str(int(v)) if ints else _num(rng, v) for v in vals)

    def shape():
        parts = []
        if rng.random() < 0.7:
            app = []
            if rng.random() < 0.8:
                if mat_defs and rng.random() < 0.3:
                    app.append(f"<Material USE={q(mat_defs[int(rng.integers(len(mat_defs)))])}/>")
                else:
                    attrs = []
                    for key in ("diffuseColor", "specularColor", "emissiveColor"):
                        if rng.random() < 0.6:
                            attrs.append(f"{key}={q(nums(rng.uniform(0, 1, 3)))}")
                    if rng.random() < 0.5:
                        attrs.append(f"shininess={q(_num(rng, rng.uniform(0, 1)))}")
                    if rng.random() < 0.3:
                        name = f"M{len(mat_defs)}"
                        mat_defs.append(name)
                        attrs.append(f"DEF={q(name)}")
                    app.append("<Material " + " ".join(attrs) + "/>")
            if rng.random() < 0.3:
                url = f"xrand{seed}.png" if rng.random() < 0.7 else "nosuch.png"
                app.append(f"<ImageTexture url={q(url)}/>")
            parts.append("<Appearance>" + "".join(app) + "</Appearance>")
        kind = rng.random()
        if kind < 0.9:
            if coord_defs and rng.random() < 0.25:
                use = list(coord_defs)[int(rng.integers(len(coord_defs)))]
                nv = coord_defs[use]
                coord = f"<Coordinate USE={q(use)}/>"
            else:
                nv = int(rng.integers(3, 30))
                dname = ""
                if rng.random() < 0.3:
                    name = f"C{len(coord_defs)}"
                    coord_defs[name] = nv
                    dname = f" DEF={q(name)}"
                coord = f"<Coordinate{dname} point={q(nums(rng.uniform(-2, 2, 3 * nv)))}/>"
            inner = [coord]
            nn = int(rng.integers(1, 20))
            nt = int(rng.integers(1, 20))
            has_n, has_t = rng.random() < 0.5, rng.random() < 0.4
            if has_n:
                inner.append(f"<Normal vector={q(nums(rng.normal(size=3 * nn)))}/>")
            if has_t:
                inner.append(f"<TextureCoordinate point={q(nums(rng.uniform(0, 1, 2 * nt)))}/>")
            if kind < 0.6:
                polys = [rng.choice(nv, int(rng.integers(3, min(5, nv) + 1)), replace=False)
                         for _ in range(int(rng.integers(1, 12)))]

                def flat(lists, trailing):
                    out = []
                    for k, p in enumerate(lists):
                        out += list(p)
                        if k + 1 < len(lists) or trailing:
                            out.append(-1)
                    return out
                attrs = [f"coordIndex={q(nums(flat(polys, rng.random() < 0.5), True))}"]
                if has_n and rng.random() < 0.6:
                    attrs.append(f"normalIndex={q(nums(flat([rng.integers(0, nn, len(p)) for p in polys], rng.random() < 0.5), True))}")
                if has_t and rng.random() < 0.6:
                    attrs.append(f"texCoordIndex={q(nums(flat([rng.integers(0, nt, len(p)) for p in polys], True), True))}")
                parts.append("<IndexedFaceSet " + " ".join(attrs) + ">" + "".join(inner) + "</IndexedFaceSet>")
            else:
                idx = rng.integers(0, nv, 3 * int(rng.integers(1, 12)))
                parts.append(f"<IndexedTriangleSet index={q(nums(idx, True))}>" + "".join(inner) +
                             "</IndexedTriangleSet>")
        return "<Shape>" + "".join(parts) + "</Shape>"

    def item(depth):
        if depth < 3 and rng.random() < 0.4:
            tag = "Transform" if rng.random() < 0.7 else "Group"
            attrs = []
            if rng.random() < 0.6:
                attrs.append(f"translation={q(nums(rng.uniform(-3, 3, 3), spaced=True))}")
            if rng.random() < 0.6:
                axis = rng.normal(size=3)
                attrs.append(f"rotation={q(nums(list(axis) + [rng.uniform(-3, 3)], spaced=True))}")
            if rng.random() < 0.5:
                attrs.append(f"scale={q(nums(rng.uniform(0.2, 3, 3), spaced=True))}")
            kids = "\n".join(item(depth + 1) for _ in range(int(rng.integers(0, 4))))
            return f"<{tag} " + " ".join(attrs) + ">\n" + kids + f"\n</{tag}>"
        if rng.random() < 0.08:
            return "<!-- skipped -->" if rng.random() < 0.5 else "<Viewpoint position='0 0 10'/>"
        return shape()

    body = "\n".join(item(0) for _ in range(int(rng.integers(1, 5))))
    name = f"xrand{seed}.x3d"
    with open(os.path.join(d, name), "w") as f:
        f.write('<?xml version="1.0" encoding="UTF-8"?>\n<X3D profile="Interchange">\n<Scene>\n' + body +
                "\n</Scene>\n</X3D>\n")
    return name
