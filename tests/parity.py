"""Shared parity checks: device path (through the C ABI) against the oracle.

Bar (per frame): visible sub-triangle id and depth bits identical, RGB8
within 1 LSB on at least 99.9% of pixels (the rest only from powf/sqrtf
rounding), float colour within 1e-4 absolute wherever the winner matches.
"""
import json
import os

import numpy as np

from minirender_gb300 import abi
from minirender_gb300.renderer import Renderer

RGB8_FRAC_MIN = 0.999
FLOAT_ATOL = 1e-4


def gpu_render(st, scene, renderer: Renderer = None, tile=None, small_max=None):
    r = renderer or Renderer(0)
    if tile is not None:
        r.ctx.set_tuning(tile, small_max if small_max is not None else 64)
    r.state = st
    r.setScene(scene)
    r.render()
    out = {"image": r.getImage(), "depth": r.getDepth(), "ids": r.getTriangleIds(),
           "rgb8": r.getImageRGB8()}
    if st.save_normals:
        out["normals"] = r.getNormalsImage()
    return out, r


def compare(gpu: dict, ref: dict, name: str = "") -> dict:
    ids_eq = np.array_equal(gpu["ids"], ref["ids"])
    depth_eq = np.array_equal(gpu["depth"].view(np.uint32), ref["depth"].view(np.uint32))
    d8 = np.abs(gpu["rgb8"].astype(np.int16) - ref["rgb8"].astype(np.int16)).max(-1)
    frac = float((d8 <= 1).mean())
    fdiff = np.abs(gpu["image"] - ref["image"])
    stats = {
        "name": name, "ids_equal": ids_eq, "depth_equal": depth_eq,
        "n_id_mismatch": int((gpu["ids"] != ref["ids"]).sum()),
        "n_depth_mismatch": int((gpu["depth"].view(np.uint32) != ref["depth"].view(np.uint32)).sum()),
        "rgb8_max_err": int(d8.max()), "rgb8_mean_err": float(d8.mean()),
        "rgb8_within_1lsb": frac, "rgb8_exact": float((d8 == 0).mean()),
        "float_max_err": float(np.nanmax(fdiff)) if fdiff.size else 0.0,
        "covered": int((ref["ids"] != abi.MR_NO_TRIANGLE).sum()),
    }
    return stats


def assert_parity(stats: dict):
    assert stats["ids_equal"], stats
    assert stats["depth_equal"], stats
    assert stats["rgb8_within_1lsb"] >= RGB8_FRAC_MIN, stats
    assert stats["float_max_err"] <= FLOAT_ATOL or stats["rgb8_max_err"] <= 1, stats


def report(stats, kind: str = "plain") -> None:
    """Appends one case's figures to parity_<kind>.jsonl in the directory named
    by MR_PARITY_REPORT_DIR (nothing is written when it is unset)."""
    d = os.environ.get("MR_PARITY_REPORT_DIR")
    if not d:
        return
    os.makedirs(d, exist_ok=True)
    rows = stats if isinstance(stats, list) else [stats]
    with open(os.path.join(d, f"parity_{kind}.jsonl"), "a") as f:
        for s in rows:
            f.write(json.dumps(s) + "\n")
