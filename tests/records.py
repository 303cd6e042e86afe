"""Decoders for the canonical per-tet records (byte layout documented in include/ria.h)."""
import struct


def decode_ia(b: bytes) -> dict:
    assert b[0] == 1
    k = b[1]
    nv, nf, nc, nloop = struct.unpack_from("<HHHH", b, 2)
    o = 10
    rep = list(b[o:o + k])
    o += k
    verts = [tuple(b[o + 3 * i:o + 3 * i + 3]) for i in range(nv)]
    o += 3 * nv
    faces = []
    for f in range(nf):
        supp, flags, pos, neg, ln = struct.unpack_from("<BBHHH", b, o + 8 * f)
        faces.append({"supp": supp, "boundary": bool(flags & 1), "pos": pos, "neg": None if neg == 0xFFFF else neg, "len": ln})
    o += 8 * nf
    for f in faces:
        f["loop"] = list(struct.unpack_from("<%dH" % f["len"], b, o))
        o += 2 * f["len"]
    cells = list(struct.unpack_from("<%dQ" % nc, b, o))
    o += 8 * nc
    assert o == len(b), (o, len(b))
    return {"k": k, "rep": rep, "verts": verts, "faces": faces, "cells": cells}


def decode_mi(b: bytes) -> dict:
    assert b[0] == 2
    k = b[1]
    nv, nf, nc, nloop = struct.unpack_from("<HHHH", b, 2)
    o = 10
    rep = list(b[o:o + k])
    o += k
    verts = [tuple(b[o + 4 * i:o + 4 * i + 4]) for i in range(nv)]
    o += 4 * nv
    faces = []
    for f in range(nf):
        pos, neg, ln = struct.unpack_from("<BBH", b, o + 4 * f)
        faces.append({"pos": pos, "neg": neg, "len": ln})
    o += 4 * nf
    for f in faces:
        f["loop"] = list(struct.unpack_from("<%dH" % f["len"], b, o))
        o += 2 * f["len"]
    cells = list(b[o:o + nc])
    o += nc
    assert o == len(b), (o, len(b))
    return {"k": k, "rep": rep, "verts": verts, "faces": faces, "cells": cells}


def split_records(rec_offsets, rec_bytes):
    """Per-tet record bytes (None for tets without a record)."""
    out = []
    for i in range(len(rec_offsets) - 1):
        a, b = int(rec_offsets[i]), int(rec_offsets[i + 1])
        out.append(bytes(rec_bytes[a:b]) if b > a else None)
    return out
