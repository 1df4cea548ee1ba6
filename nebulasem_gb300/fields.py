"""Reference field files: read and write `<name><step>.bin` / `.txt`.

Format of NebulaSEM's MeshField::write (src/field/field.h:1589-1677) through
its binary stream (src/util/util.h:191-258): strings are written without
whitespace as a one-byte length and the bytes, integers (`Int`, unsigned
32-bit) and scalars (double) as raw little-endian values:

    "size" <Int components> "internal" <Int count> "{" <count x components doubles> "}"
    "boundary" <Int n> "{" <n boundary blocks> "}"

The text form has the same tokens separated by whitespace, values printed with
12 significant digits (lossy).  Only explicit internal values are read here
(count > 4; the reference's initialisers such as `uniform` or `cosine` are
expressions it evaluates on its mesh).  The boundary section is kept as raw
bytes (binary) or text so that a written file carries the original boundary
conditions unchanged.
"""
import re
import struct

import numpy as np


class FieldFile:
    """Internal values (count x components, float64) and the boundary section."""

    def __init__(self, values, boundary=b"", binary=True):
        self.values = np.ascontiguousarray(np.asarray(values, dtype=np.float64))
        if self.values.ndim == 1:
            self.values = self.values[:, None]
        self.boundary = boundary
        self.binary = binary

    @property
    def components(self):
        return self.values.shape[1]


def _read_str(buf, pos):
    n = buf[pos]
    return buf[pos + 1:pos + 1 + n].decode(), pos + 1 + n


def _write_str(s):
    s = "".join(s.split())
    b = s.encode()
    return bytes([len(b)]) + b if b else b""


def read_field(path):
    """Read a reference field file (.bin or .txt) with explicit internal values."""
    if path.endswith(".bin"):
        buf = open(path, "rb").read()
        tok, pos = _read_str(buf, 0)
        if tok != "size":
            raise ValueError(f"{path}: expected 'size', found {tok!r}")
        (ncomp,), pos = struct.unpack_from("<I", buf, pos), pos + 4
        tok, pos = _read_str(buf, pos)
        if tok != "internal":
            raise ValueError(f"{path}: internal field not found")
        (count,), pos = struct.unpack_from("<I", buf, pos), pos + 4
        tok, pos = _read_str(buf, pos)
        if tok != "{":
            raise ValueError(f"{path}: expected '{{'")
        if count <= 4:
            raise ValueError(f"{path}: initialiser expressions are not values")
        nval = count * ncomp
        vals = np.frombuffer(buf, dtype="<f8", count=nval, offset=pos).reshape(count, ncomp)
        pos += 8 * nval
        tok, pos = _read_str(buf, pos)
        if tok != "}":
            raise ValueError(f"{path}: expected '}}'")
        return FieldFile(vals.copy(), buf[pos:], binary=True)
    text = open(path).read()
    spans = [(m.group(), m.end()) for m in re.finditer(r"\S+", text)]
    toks = [t for t, _ in spans]
    if toks[0] != "size" or toks[2] != "internal" or toks[4] != "{":
        raise ValueError(f"{path}: not a field file with explicit values")
    ncomp, count = int(toks[1]), int(toks[3])
    if count <= 4:
        raise ValueError(f"{path}: initialiser expressions are not values")
    nval = count * ncomp
    vals = np.array([float(t) for t in toks[5:5 + nval]]).reshape(count, ncomp)
    if toks[5 + nval] != "}":
        raise ValueError(f"{path}: expected '}}'")
    # boundary section: the text after the internal block's closing brace
    return FieldFile(vals, text[spans[5 + nval][1]:].lstrip("\n"), binary=False)


def write_field(path, ff):
    """Write a FieldFile in the binary (.bin) or text (.txt) form of its path."""
    count, ncomp = ff.values.shape
    if path.endswith(".bin"):
        out = bytearray()
        out += _write_str("size") + struct.pack("<I", ncomp)
        out += _write_str("internal") + struct.pack("<I", count) + _write_str("{")
        out += ff.values.astype("<f8").tobytes()
        out += _write_str("}")
        boundary = ff.boundary if isinstance(ff.boundary, (bytes, bytearray)) else \
            _write_str("boundary") + struct.pack("<I", 0) + _write_str("{") + _write_str("}")
        out += boundary
        with open(path, "wb") as f:
            f.write(bytes(out))
        return
    lines = [f"size {ncomp}", f"internal {count}", "{"]
    for row in ff.values:
        lines.append(" ".join(repr(float(x)) for x in row) + (" " if ncomp > 1 else ""))
    lines.append("}")
    boundary = ff.boundary if isinstance(ff.boundary, str) else "boundary 0\n{\n}\n"
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n" + boundary)
