"""Save/load of a golden case: the scene (pre-order node array, meshes,
textures), the renderer state and the reference outputs, in one .npz."""
import numpy as np

from minirender_gb300.frame import FrameState
from minirender_gb300.scene import Material, Scene, SceneNode, TriMesh
from minirender_gb300 import scene as S

_FRAME_KEYS = ["width", "height", "projection", "view", "light", "light_is_point", "ambient",
               "background", "lighting", "texturing", "save_normals"]


def save_case(path, st: FrameState, scene, expect: dict):
    flat = S.flatten(scene)
    d = {}
    f = st.to_c()
    d["frame_wh"] = np.array([f.width, f.height], np.int32)
    d["frame_proj"] = np.array(f.projection[:], np.float32)
    d["frame_view"] = np.array(f.view[:], np.float32)
    d["frame_light"] = np.array(f.light[:], np.float32)
    d["frame_bg"] = np.array(f.background[:], np.float32)
    d["frame_flags"] = np.array([f.light_is_point, f.lighting, f.texturing, f.save_normals], np.int32)
    d["frame_ambient"] = np.array([f.ambient], np.float32)
    nodes = flat.nodes
    d["node_parent"] = np.array([n.parent for n in nodes], np.int32)
    d["node_mesh"] = np.array([n.mesh for n in nodes], np.int32)
    d["node_xf"] = np.array([n.transform[:] for n in nodes], np.float32)
    d["node_hasmat"] = np.array([n.has_material for n in nodes], np.int32)
    d["node_mat"] = np.array([list(n.material.diffuse) + list(n.material.specular) +
                              list(n.material.emissive) + [n.material.shininess] for n in nodes], np.float32)
    d["node_tex"] = np.array([n.material.texture for n in nodes], np.int32)
    for i, m in enumerate(flat.meshes):
        for k in ("vertices", "normals", "texcoords", "indices", "normalsI", "texcoordsI"):
            d[f"mesh{i}_{k}"] = getattr(m, k)
    d["n_meshes"] = np.array([len(flat.meshes)], np.int32)
    for i, t in enumerate(flat.textures):
        d[f"tex{i}"] = t
    d["n_tex"] = np.array([len(flat.textures)], np.int32)
    for k, v in expect.items():
        d["expect_" + k] = v
    np.savez_compressed(path, **d)


def load_case(path):
    z = np.load(path)
    wh = z["frame_wh"]
    flags = z["frame_flags"]
    st = FrameState(width=int(wh[0]), height=int(wh[1]), projection=z["frame_proj"].reshape(4, 4),
                    view=z["frame_view"].reshape(4, 4), light=z["frame_light"],
                    light_is_point=bool(flags[0]), ambient=float(z["frame_ambient"][0]),
                    background=z["frame_bg"], lighting=bool(flags[1]), texturing=bool(flags[2]),
                    save_normals=bool(flags[3]))
    texs = [z[f"tex{i}"] for i in range(int(z["n_tex"][0]))]
    meshes = []
    for i in range(int(z["n_meshes"][0])):
        g = lambda k: z[f"mesh{i}_{k}"]  # noqa: E731
        meshes.append(dict(vertices=g("vertices"), normals=g("normals"), indices=g("indices"),
                           normalsI=g("normalsI"), texcoords=g("texcoords"), texcoordsI=g("texcoordsI")))
    parents = z["node_parent"]
    built = []
    scene = None
    for i in range(parents.size):
        mi = int(z["node_mesh"][i])
        if i == 0:
            node = Scene()
            node.ambientLight = np.float32(z["frame_ambient"][0])
            scene = node
        elif mi >= 0:
            m = meshes[mi]
            mat = None
            if z["node_hasmat"][i]:
                mv = z["node_mat"][i]
                t = int(z["node_tex"][i])
                mat = Material(diffuse=mv[0:3], specular=mv[3:6], emissive=mv[6:9], shininess=mv[9],
                               texture=texs[t] if t >= 0 else None)
            node = TriMesh(m["vertices"], m["normals"], m["indices"], normalsI=m["normalsI"],
                           texcoords=m["texcoords"] if m["texcoords"].size else None,
                           texcoordsI=m["texcoordsI"] if m["texcoordsI"].size else None, material=mat)
        else:
            node = SceneNode()
        node.transform = z["node_xf"][i].reshape(4, 4).copy()
        if i > 0:
            built[int(parents[i])].add(node)
        built.append(node)
    expect = {k[len("expect_"):]: z[k] for k in z.files if k.startswith("expect_")}
    return st, scene, expect
