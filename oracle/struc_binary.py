"""Restatement of the reference's binary structure file (Structure::write_binary/read_binary,
src/struc/structure.cpp:117-190) in plain Python, as a checker of the C++ reader and writer.

TEST INFRASTRUCTURE ONLY: used by the tests as the checker, never by the product.  Parity
status: no binary file written by the reference exists here (the reference cannot be built), so
the layout is pinned by reading the reference's serialize code, cited per record below.

A file is an int byte count followed by serialize::pack(Structure) (structure.cpp:643-649):
  Cell      pack(Eigen::Matrix3d): 9 doubles, column-major (cell.cpp:190-194, eigen.cpp:75)
  State     energy ewald temp press qtot pe ke dt as doubles, t as int (state.cpp:67-79)
  AtomData  pack(AtomType): 16 bools (atom_type.cpp:124-147; frac is not written), int natoms,
            then the flagged properties in the order of structure.cpp:610-642:
              name            int count, (int length, chars) each (serialize.cpp:70-79)
              an type index   int count, ints (serialize.cpp:80-88)
              mass ... js     int count, doubles (serialize.cpp:98-106)
              posn vel force spin  int count, 3 doubles each (eigen.cpp:87-95)
              symm            int count, (int size, doubles) each (eigen.cpp:66-74,96-102)
Byte order is the machine's (little-endian on both hosts used here).
"""
import struct

import numpy as np

FLAGS = ["name", "an", "type", "index", "mass", "charge", "radius", "chi", "eta", "c6", "js",
         "posn", "vel", "force", "spin", "symm"]
STATE = ["energy", "ewald", "temp", "press", "qtot", "pe", "ke", "dt"]
INTS = ("an", "type", "index")
DOUBLES = ("mass", "charge", "radius", "chi", "eta", "c6", "js")
VEC3 = ("posn", "vel", "force", "spin")


def pack(s):
    """Bytes of a structure given as a dict: R (3x3, columns = lattice vectors), the STATE keys
    and t, flags (dict name -> bool) and one array per flagged property."""
    out = [np.asarray(s["R"], np.float64).reshape(3, 3).flatten(order="F").tobytes()]
    out.append(struct.pack("<8d", *[float(s.get(k, 0.0)) for k in STATE]))
    out.append(struct.pack("<i", int(s.get("t", 0))))
    flags = s["flags"]
    out.append(bytes(1 if flags.get(f, False) else 0 for f in FLAGS))
    n = int(s["natoms"])
    out.append(struct.pack("<i", n))
    for f in FLAGS:
        if not flags.get(f, False):
            continue
        v = s[f]
        if f == "name":
            out.append(struct.pack("<i", len(v)))
            for nm in v:
                b = nm.encode()
                out.append(struct.pack("<i", len(b)) + b)
        elif f in INTS:
            a = np.asarray(v, np.int32)
            out.append(struct.pack("<i", len(a)) + a.tobytes())
        elif f in DOUBLES:
            a = np.asarray(v, np.float64)
            out.append(struct.pack("<i", len(a)) + a.tobytes())
        elif f in VEC3:
            a = np.asarray(v, np.float64).reshape(-1, 3)
            out.append(struct.pack("<i", len(a)) + a.tobytes())
        else:  # symm
            out.append(struct.pack("<i", len(v)))
            for g in v:
                a = np.asarray(g, np.float64)
                out.append(struct.pack("<i", len(a)) + a.tobytes())
    body = b"".join(out)
    return struct.pack("<i", len(body)) + body


def unpack(data):
    """The dict pack() takes, from the bytes of a file."""
    (nbytes,) = struct.unpack_from("<i", data, 0)
    assert nbytes == len(data) - 4, "byte count does not match the file"
    pos = 4
    s = {"R": np.frombuffer(data, np.float64, 9, pos).reshape(3, 3, order="F").copy()}
    pos += 72
    for k, v in zip(STATE, struct.unpack_from("<8d", data, pos)):
        s[k] = v
    pos += 64
    (s["t"],) = struct.unpack_from("<i", data, pos)
    pos += 4
    s["flags"] = {f: data[pos + k] != 0 for k, f in enumerate(FLAGS)}
    pos += 16
    (s["natoms"],) = struct.unpack_from("<i", data, pos)
    pos += 4

    def count():
        nonlocal pos
        (c,) = struct.unpack_from("<i", data, pos)
        pos += 4
        return c

    for f in FLAGS:
        if not s["flags"][f]:
            continue
        c = count()
        if f == "name":
            names = []
            for _ in range(c):
                ln = count()
                names.append(data[pos:pos + ln].decode())
                pos += ln
            s[f] = names
        elif f in INTS:
            s[f] = np.frombuffer(data, np.int32, c, pos).copy()
            pos += 4 * c
        elif f in DOUBLES:
            s[f] = np.frombuffer(data, np.float64, c, pos).copy()
            pos += 8 * c
        elif f in VEC3:
            s[f] = np.frombuffer(data, np.float64, 3 * c, pos).reshape(c, 3).copy()
            pos += 24 * c
        else:
            rows = []
            for _ in range(c):
                ln = count()
                rows.append(np.frombuffer(data, np.float64, ln, pos).copy())
                pos += 8 * ln
            s[f] = rows
    assert pos == len(data), "trailing bytes"
    return s
