"""Test infrastructure: a plain-Python restatement of the reference's .osh
binary format (src/Omega_h_file.cpp), used as the checker for the library's
device-resident .osh reader and writer.  Not part of the product.

Layout of ``<dir>/0.osh`` (one part), all values little endian:

* magic 0xa1 0x1a; I8 is_compressed (src/Omega_h_file.cpp:355-366);
* meta (write_meta/read_meta, :200-272): I8 family (version >= 7), I8 dim,
  I32 comm size, I32 comm rank, I8 parting, I32 ghost layers (version >= 3),
  I8 have_hints (+ I32 naxes, 3 Reals each), I8 keeps_canon (version < 6);
* LO nverts; for d = 1..dim: the down adjacency ab2b, and its codes for d > 1
  (:367-373);
* for d = 0..dim: I32 ntags, then each tag (write_tag/read_tag, :274-332):
  string name (I32 length + bytes), I8 ncomps, I8 type (0 I8, 2 I32, 3 I64,
  5 F64), (version < 5: I8 xfer, version >= 2 also I8 outflags), array;
* I32 nsets; each: name, I32 npairs, pairs of (I32 dim, I32 id) (:334-356),
  version >= 8;
* I8 has_parents (version >= 9), then per dimension parent_idx and codes.

An array (write_array/read_array, :117-176) is LO size, then either the raw
bytes or (compressed) I64 compressed size and a zlib stream.
``<dir>/nparts`` and ``<dir>/version`` hold one integer each (:470-486).
"""
import os
import struct
import zlib

import numpy as np

MAGIC = b"\xa1\x1a"
LATEST_VERSION = 9
TYPES = {0: np.int8, 2: np.int32, 3: np.int64, 5: np.float64}


class _Reader:
    def __init__(self, b):
        self.b, self.p = b, 0

    def val(self, fmt):
        v = struct.unpack_from("<" + fmt, self.b, self.p)[0]
        self.p += struct.calcsize("<" + fmt)
        return v

    def raw(self, n):
        out = self.b[self.p:self.p + n]
        assert len(out) == n, "truncated file"
        self.p += n
        return out

    def string(self):
        return self.raw(self.val("i")).decode()

    def array(self, dtype, compressed):
        n = self.val("i")
        assert n >= 0
        nbytes = n * np.dtype(dtype).itemsize
        if compressed:
            data = zlib.decompress(self.raw(self.val("q")))
            assert len(data) == nbytes
        else:
            data = self.raw(nbytes)
        return np.frombuffer(data, dtype=np.dtype(dtype).newbyteorder("<")).copy()


def read(path):
    """The mesh of an .osh directory as a dict."""
    with open(os.path.join(path, "nparts")) as f:
        assert int(f.read().split()[0]) == 1, "one part only"
    with open(os.path.join(path, "version")) as f:
        version = int(f.read().split()[0])
    with open(os.path.join(path, "0.osh"), "rb") as f:
        r = _Reader(f.read())
    assert r.raw(2) == MAGIC
    assert 1 <= version <= LATEST_VERSION
    m = {"version": version}
    comp = r.val("b")
    m["compressed"] = comp
    m["family"] = r.val("b") if version >= 7 else 0
    m["dim"] = dim = r.val("b")
    m["comm_size"], m["comm_rank"] = r.val("i"), r.val("i")
    m["parting"] = r.val("b")
    m["nghost_layers"] = r.val("i") if version >= 3 else 0
    hints = r.val("b")
    m["hints"] = [[r.val("d") for _ in range(3)] for _ in range(r.val("i"))] if hints else None
    if version < 6:
        r.val("b")
    m["nverts"] = r.val("i")
    m["down"], m["codes"] = {}, {}
    for d in range(1, dim + 1):
        m["down"][d] = r.array(np.int32, comp)
        if d > 1:
            m["codes"][d] = r.array(np.int8, comp)
    m["tags"] = {}
    for d in range(dim + 1):
        tags = []
        for _ in range(r.val("i")):
            name = r.string()
            ncomps, ty = r.val("b"), r.val("b")
            if version < 5:
                r.val("b")
                if version >= 2:
                    r.val("b")
            tags.append((name, ncomps, ty, r.array(TYPES[ty], comp)))
        m["tags"][d] = tags
    m["sets"] = []
    if version >= 8:
        for _ in range(r.val("i")):
            name = r.string()
            m["sets"].append((name, [(r.val("i"), r.val("i")) for _ in range(r.val("i"))]))
    m["has_parents"] = r.val("b") if version >= 9 else 0
    assert not m["has_parents"], "parents not modelled here"
    assert r.p == len(r.b), "trailing bytes"
    return m


def _array(out, a, compressed, level=1):
    a = np.ascontiguousarray(a)
    out.append(struct.pack("<i", a.size))
    data = a.astype(a.dtype.newbyteorder("<")).tobytes()
    if compressed:
        z = zlib.compress(data, level)
        out.append(struct.pack("<q", len(z)))
        out.append(z)
    else:
        out.append(data)


def write(path, m):
    """Write a mesh dict (as ``read`` returns) in the latest version."""
    out = [MAGIC, struct.pack("<b", m["compressed"])]
    out.append(struct.pack("<bbiibib", m["family"], m["dim"], m["comm_size"], m["comm_rank"],
                           m["parting"], m["nghost_layers"], 1 if m["hints"] else 0))
    if m["hints"]:
        out.append(struct.pack("<i", len(m["hints"])))
        for ax in m["hints"]:
            out.append(struct.pack("<ddd", *ax))
    out.append(struct.pack("<i", m["nverts"]))
    for d in range(1, m["dim"] + 1):
        _array(out, m["down"][d], m["compressed"])
        if d > 1:
            _array(out, m["codes"][d], m["compressed"])
    for d in range(m["dim"] + 1):
        out.append(struct.pack("<i", len(m["tags"][d])))
        for name, ncomps, ty, a in m["tags"][d]:
            out.append(struct.pack("<i", len(name)) + name.encode())
            out.append(struct.pack("<bb", ncomps, ty))
            _array(out, a, m["compressed"])
    out.append(struct.pack("<i", len(m["sets"])))
    for name, pairs in m["sets"]:
        out.append(struct.pack("<i", len(name)) + name.encode())
        out.append(struct.pack("<i", len(pairs)))
        for d, i in pairs:
            out.append(struct.pack("<ii", d, i))
    out.append(struct.pack("<b", 0))
    os.makedirs(path, exist_ok=True)
    with open(os.path.join(path, "0.osh"), "wb") as f:
        f.write(b"".join(out))
    for name, v in (("nparts", 1), ("version", LATEST_VERSION)):
        with open(os.path.join(path, name), "w") as f:
            f.write(f"{v}\n")


def tag(m, d, name):
    for t in m["tags"][d]:
        if t[0] == name:
            return t[3]
    raise KeyError(f"no tag {name} on dimension {d}")


def compare(a, b, rtol=1e-12):
    """Differences between two mesh dicts: metadata, connectivity, tag names,
    orders and integer arrays exactly; reals within rtol.  Returns a list of
    messages (empty when they agree)."""
    bad = []
    for k in ("family", "dim", "comm_size", "comm_rank", "parting", "nghost_layers", "hints",
              "nverts", "sets", "has_parents"):
        if a[k] != b[k]:
            bad.append(f"{k}: {a[k]} vs {b[k]}")
    for key in ("down", "codes"):
        for d in a[key]:
            if not np.array_equal(a[key][d], b[key].get(d)):
                bad.append(f"{key}[{d}] differs")
    for d in a["tags"]:
        na = [(t[0], t[1], t[2]) for t in a["tags"][d]]
        nb = [(t[0], t[1], t[2]) for t in b["tags"][d]]
        if na != nb:
            bad.append(f"tags of dimension {d}: {na} vs {nb}")
            continue
        for (name, _, ty, x), (_, _, _, y) in zip(a["tags"][d], b["tags"][d]):
            if x.shape != y.shape:
                bad.append(f"{name}@{d}: size {x.size} vs {y.size}")
            elif ty == 5:
                den = np.maximum(np.abs(x), np.abs(y))
                err = np.abs(x - y) / np.where(den > 0, den, 1.0)
                if err.size and err.max() > rtol:
                    bad.append(f"{name}@{d}: max relative error {err.max():.3e}")
            elif not np.array_equal(x, y):
                bad.append(f"{name}@{d}: {int(np.sum(x != y))} entries differ")
    return bad
