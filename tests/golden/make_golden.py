"""Regenerate the golden fixtures in this folder.

Run from the repository root with the path of the reference checkout (it
reads the reference's own test asset; nothing at test time reads it):

    python tests/golden/make_golden.py <reference checkout>

Writes kitchen_mesh.npz: the triangles of assets/kitchen.obj.zst as loaded by
examples/helpers/load_obj.rs:6-45 (positions as f32, faces in file order,
quads split (a,b,c),(a,c,d)), stored as deduplicated vertex positions plus a
face index table.  examples/obj_cwbvh.rs:142-181 renders this mesh at 32x18
and asserts the normal hash 1343358762 for five build presets.
"""
from __future__ import annotations

import argparse
import ctypes
import os

import numpy as np

#: the mesh inside the reference checkout
ASSET = os.path.join("assets", "kitchen.obj.zst")
HERE = os.path.dirname(os.path.abspath(__file__))


class _Buf(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("size", ctypes.c_size_t), ("pos", ctypes.c_size_t)]


def zstd_decompress(data: bytes) -> bytes:
    """Streaming decompression through the system libzstd (frame size unknown)."""
    z = ctypes.CDLL("libzstd.so.1")
    z.ZSTD_createDStream.restype = ctypes.c_void_p
    z.ZSTD_decompressStream.restype = ctypes.c_size_t
    z.ZSTD_isError.restype = ctypes.c_uint
    ds = z.ZSTD_createDStream()
    z.ZSTD_initDStream(ctypes.c_void_p(ds))
    src = ctypes.create_string_buffer(data, len(data))
    inb = _Buf(ctypes.cast(src, ctypes.c_void_p), len(data), 0)
    cap = 1 << 20
    chunk = ctypes.create_string_buffer(cap)
    out = []
    try:
        while True:
            outb = _Buf(ctypes.cast(chunk, ctypes.c_void_p), cap, 0)
            r = z.ZSTD_decompressStream(ctypes.c_void_p(ds), ctypes.byref(outb), ctypes.byref(inb))
            if z.ZSTD_isError(r):
                raise RuntimeError("zstd decompression failed")
            out.append(chunk.raw[: outb.pos])
            if inb.pos == inb.size and outb.pos < cap:
                break
    finally:
        z.ZSTD_freeDStream(ctypes.c_void_p(ds))
    return b"".join(out)


def load_obj_triangles(text: str) -> np.ndarray:
    pos = []
    tris = []
    for line in text.splitlines():
        if line.startswith("v "):
            pos.append([np.float32(x) for x in line.split()[1:4]])
        elif line.startswith("f "):
            idx = [int(t.split("/")[0]) for t in line.split()[1:]]
            idx = [i - 1 if i > 0 else len(pos) + i for i in idx]
            tris.append(pos[idx[0]] + pos[idx[1]] + pos[idx[2]])
            if len(idx) == 4:
                tris.append(pos[idx[0]] + pos[idx[2]] + pos[idx[3]])
    return np.array(tris, np.float32)


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("reference", help="path of the obvhs reference checkout")
    args = ap.parse_args()
    text = zstd_decompress(open(os.path.join(args.reference, ASSET), "rb").read()).decode()
    tris = load_obj_triangles(text)
    verts = tris.reshape(-1, 3)
    uniq, inv = np.unique(verts.view(np.uint32).reshape(-1, 3), axis=0, return_inverse=True)
    faces = inv.reshape(-1, 3).astype(np.uint32)
    np.savez_compressed(os.path.join(HERE, "kitchen_mesh.npz"), positions=uniq.view(np.float32), faces=faces)
    print(f"kitchen: {len(tris)} triangles, {len(uniq)} unique positions")


if __name__ == "__main__":
    main()
