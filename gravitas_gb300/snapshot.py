"""Reading and writing .gravitas snapshots (internal/save/save.go).

A snapshot is a gzip-compressed encoding/gob stream holding one save.File value (save.go:38-67):
run metadata, sim.Params, the body arrays (PosX..VelZ, Mass, Kind, ...) and the last force
evaluation (*sim.Forces) for an exact continuation. This module restates the gob wire format
(Go's published encoding/gob specification) in Python:

  unsigned ints   < 128 in one byte, else the negated byte count, then big-endian bytes
  signed ints     zig-zag: i >= 0 -> i << 1, i < 0 -> (~i << 1) | 1, then as unsigned
  floats          the IEEE-754 bits byte-reversed, then as unsigned
  strings, bytes  length, then the bytes (every slice of a uint8 kind travels as bytes)
  structs         (field-number delta, value) pairs, zero values omitted, terminated by 0
  slices, arrays  element count, then the elements; maps: count, then key/value pairs
  messages        byte count, then a type id (negative: a wireType definition follows) and
                  the value; non-struct top-level values start with a 0 delta

`read` decodes any gob stream generically (structs become dicts keyed by field name, float and
int slices numpy arrays, GobEncoder values such as time.Time their raw bytes), so a snapshot
written by the reference with all its fields (Scene, Camera, gas, radiation, spins) reads, and
`load_state` extracts the bodies and forces the force and step path needs. `save` writes a
File value with the fields this library owns (Format, Params, Time, Steps, the body arrays and
Forces); gob matches struct fields by name, so the reference's reader takes it and leaves the
other fields zero.
"""
from __future__ import annotations

import gzip
import io
import struct as _struct

import numpy as np

FORMAT = 4            # save.go:21
EXTENSION = ".gravitas"


class GobError(ValueError):
    """A malformed or unsupported gob stream."""


# ---- built-in type ids (encoding/gob type.go) ----
T_BOOL, T_INT, T_UINT, T_FLOAT, T_BYTES, T_STRING, T_COMPLEX, T_INTERFACE = 1, 2, 3, 4, 5, 6, 7, 8
FIRST_USER_ID = 65


# ---- primitive encodings ----

def enc_uint(x: int) -> bytes:
    if x < 0:
        raise GobError("negative unsigned")
    if x < 128:
        return bytes([x])
    b = x.to_bytes((x.bit_length() + 7) // 8, "big")
    return bytes([(256 - len(b)) & 0xFF]) + b


def enc_int(i: int) -> bytes:
    return enc_uint((~i << 1) | 1 if i < 0 else i << 1)


def enc_float(f: float) -> bytes:
    bits = int.from_bytes(_struct.pack("<d", f), "big")  # the little-endian bytes read big-endian: reversed
    return enc_uint(bits)


def enc_bytes(b: bytes) -> bytes:
    return enc_uint(len(b)) + bytes(b)


class _In:
    def __init__(self, data: bytes):
        self.d, self.p = data, 0

    def byte(self) -> int:
        if self.p >= len(self.d):
            raise GobError("unexpected end of data")
        b = self.d[self.p]
        self.p += 1
        return b

    def take(self, n: int) -> bytes:
        if n < 0 or self.p + n > len(self.d):
            raise GobError("unexpected end of data")
        b = self.d[self.p:self.p + n]
        self.p += n
        return b

    def uint(self) -> int:
        b = self.byte()
        if b < 128:
            return b
        n = 256 - b
        if n > 8:
            raise GobError(f"bad unsigned length {n}")
        return int.from_bytes(self.take(n), "big")

    def int(self) -> int:
        u = self.uint()
        return ~(u >> 1) if u & 1 else u >> 1

    def float(self) -> float:
        u = self.uint()
        if u >= 1 << 64:
            raise GobError("float out of range")
        return _struct.unpack("<d", u.to_bytes(8, "big"))[0]

    def bytes(self) -> bytes:
        return self.take(self.uint())

    def done(self) -> bool:
        return self.p >= len(self.d)


# ---- types ----

class GType:
    """A gob type: kind 'struct' (fields: list of (name, GType)), 'slice' / 'array' (elem, n),
    'map' (key, elem), 'gob' (an externally encoded value: bytes) or a built-in id."""

    def __init__(self, kind, name="", fields=None, elem=None, key=None, length=0, builtin=0):
        self.kind, self.name, self.fields = kind, name, fields or []
        self.elem, self.key, self.length, self.builtin = elem, key, length, builtin


BOOL, INT, UINT, FLOAT = (GType("builtin", builtin=t) for t in (T_BOOL, T_INT, T_UINT, T_FLOAT))
BYTES, STRING = GType("builtin", builtin=T_BYTES), GType("builtin", builtin=T_STRING)


def Struct(name, fields):
    return GType("struct", name=name, fields=fields)


def Slice(elem):
    return BYTES if elem is BYTES else GType("slice", elem=elem)


def Array(elem, n):
    return GType("array", elem=elem, length=n)


def Map(key, elem):
    return GType("map", key=key, elem=elem)


def Encoded(name):
    """A GobEncoder / BinaryMarshaler value (for instance time.Time): raw bytes."""
    return GType("gob", name=name)


# ---- encoder ----

class Encoder:
    """Encodes values of GType schemas into one gob stream (type definitions sent once)."""

    def __init__(self):
        self.out = io.BytesIO()
        self.ids: dict[int, int] = {}
        self.next_id = FIRST_USER_ID

    def _id(self, t: GType) -> int:
        if t.kind == "builtin":
            return t.builtin
        key = id(t)
        if key in self.ids:
            return self.ids[key]
        tid = self.next_id
        self.next_id += 1
        self.ids[key] = tid
        # component types first, so every id a definition names is defined before a value uses it
        comps = [f for _, f in t.fields] if t.kind == "struct" else [c for c in (t.elem, t.key) if c is not None]
        comp_ids = [self._id(c) for c in comps]
        common = self._common(t.name, tid)
        if t.kind == "struct":
            fields = b"".join(b"\x01" + enc_bytes(n.encode()) + b"\x01" + enc_int(i) + b"\x00"
                              for (n, _), i in zip(t.fields, comp_ids))
            body = b"\x03" + b"\x01" + common + b"\x01" + enc_uint(len(t.fields)) + fields + b"\x00"
        elif t.kind == "slice":
            body = b"\x02" + b"\x01" + common + b"\x01" + enc_int(comp_ids[0]) + b"\x00"
        elif t.kind == "array":
            body = b"\x01" + b"\x01" + common + b"\x01" + enc_int(comp_ids[0]) + b"\x01" + enc_int(t.length) + b"\x00"
        elif t.kind == "map":
            body = b"\x04" + b"\x01" + common + b"\x01" + enc_int(comp_ids[1]) + b"\x01" + enc_int(comp_ids[0]) + b"\x00"
        elif t.kind == "gob":
            body = b"\x05" + b"\x01" + common + b"\x00"
        else:
            raise GobError(f"cannot define {t.kind}")
        self._message(enc_int(-tid) + body + b"\x00")
        return tid

    @staticmethod
    def _common(name: str, tid: int) -> bytes:
        c = b""
        if name:
            c += b"\x01" + enc_bytes(name.encode())
        return c + (b"\x02" if not name else b"\x01") + enc_int(tid) + b"\x00"

    def _message(self, payload: bytes):
        self.out.write(enc_uint(len(payload)) + payload)

    def _zero(self, t: GType, v) -> bool:
        if v is None:
            return True
        if t.kind == "builtin":
            if t.builtin in (T_BYTES, T_STRING):
                return len(v) == 0
            return v == 0 or v is False
        if t.kind in ("slice", "map"):
            return len(v) == 0
        if t.kind == "struct":
            return all(self._zero(ft, v.get(fn)) for fn, ft in t.fields)
        if t.kind == "gob":
            return False
        return False

    def _value(self, t: GType, v) -> bytes:
        if t.kind == "builtin":
            b = t.builtin
            if b == T_BOOL:
                return enc_uint(1 if v else 0)
            if b == T_INT:
                return enc_int(int(v))
            if b == T_UINT:
                return enc_uint(int(v))
            if b == T_FLOAT:
                return enc_float(float(v))
            if b == T_BYTES:
                return enc_bytes(bytes(np.asarray(v, np.uint8).tobytes() if not isinstance(v, (bytes, bytearray)) else v))
            if b == T_STRING:
                return enc_bytes(v.encode())
            raise GobError(f"cannot encode built-in {b}")
        if t.kind == "struct":
            out, last = b"", -1
            for k, (fn, ft) in enumerate(t.fields):
                fv = v.get(fn) if isinstance(v, dict) else None
                if self._zero(ft, fv):
                    continue
                out += enc_uint(k - last) + self._value(ft, fv)
                last = k
            return out + b"\x00"
        if t.kind == "slice":
            return enc_uint(len(v)) + b"".join(self._value(t.elem, x) for x in v)
        if t.kind == "array":
            if len(v) != t.length:
                raise GobError("array length")
            return enc_uint(len(v)) + b"".join(self._value(t.elem, x) for x in v)
        if t.kind == "map":
            return enc_uint(len(v)) + b"".join(self._value(t.key, k) + self._value(t.elem, x) for k, x in v.items())
        if t.kind == "gob":
            return enc_bytes(bytes(v))
        raise GobError(f"cannot encode {t.kind}")

    def encode(self, t: GType, v) -> "Encoder":
        tid = self._id(t)
        body = self._value(t, v)
        if t.kind != "struct":
            body = b"\x00" + body  # singleton: a zero field delta
        self._message(enc_int(tid) + body)
        return self

    def getvalue(self) -> bytes:
        return self.out.getvalue()


# ---- decoder ----

class Decoder:
    """Decodes a gob stream: wire-type definitions into GTypes, values into Python objects."""

    def __init__(self, data: bytes):
        self.inp = _In(data)
        self.types: dict[int, GType] = {}

    def _wire_common(self, r: _In):
        name, tid, f = "", 0, -1
        while True:
            d = r.uint()
            if d == 0:
                return name, tid
            f += d
            if f == 0:
                name = r.bytes().decode()
            elif f == 1:
                tid = r.int()
            else:
                raise GobError("bad CommonType")

    def _wire_type(self, r: _In) -> GType:
        f, t = -1, None
        while True:
            d = r.uint()
            if d == 0:
                break
            f += d
            sub, name, elem, key, length, fields = -1, "", 0, 0, 0, []
            while True:
                dd = r.uint()
                if dd == 0:
                    break
                sub += dd
                if sub == 0:
                    name, _ = self._wire_common(r)
                elif f == 2 and sub == 1:  # structType.Field
                    for _ in range(r.uint()):
                        fn, fid, ff = "", 0, -1
                        while True:
                            d3 = r.uint()
                            if d3 == 0:
                                break
                            ff += d3
                            if ff == 0:
                                fn = r.bytes().decode()
                            elif ff == 1:
                                fid = r.int()
                            else:
                                raise GobError("bad fieldType")
                        fields.append((fn, fid))
                elif f in (0, 1, 3) and sub == 1:
                    v = r.int()
                    if f == 3:
                        key = v
                    else:
                        elem = v
                elif f == 0 and sub == 2:
                    length = r.int()
                elif f == 3 and sub == 2:
                    elem = r.int()
                else:
                    raise GobError(f"bad wireType field {f}.{sub}")
            if f == 0:
                t = GType("array", name=name, elem=elem, length=length)
            elif f == 1:
                t = GType("slice", name=name, elem=elem)
            elif f == 2:
                t = GType("struct", name=name, fields=fields)
            elif f == 3:
                t = GType("map", name=name, key=key, elem=elem)
            elif f in (4, 5, 6):
                t = GType("gob", name=name)
            else:
                raise GobError(f"unknown wireType field {f}")
        if t is None:
            raise GobError("empty wireType")
        return t

    def _value(self, tid: int, r: _In):
        if tid == T_BOOL:
            return r.uint() != 0
        if tid == T_INT:
            return r.int()
        if tid == T_UINT:
            return r.uint()
        if tid == T_FLOAT:
            return r.float()
        if tid == T_BYTES:
            return r.bytes()
        if tid == T_STRING:
            return r.bytes().decode()
        if tid == T_COMPLEX:
            return complex(r.float(), r.float())
        if tid == T_INTERFACE:
            return self._interface(r)
        t = self.types.get(tid)
        if t is None:
            raise GobError(f"undefined type id {tid}")
        if t.kind == "struct":
            out, f = {}, -1
            while True:
                d = r.uint()
                if d == 0:
                    return out
                f += d
                if f >= len(t.fields):
                    raise GobError("field number out of range")
                fn, fid = t.fields[f]
                out[fn] = self._value(fid, r)
        if t.kind in ("slice", "array"):
            n = r.uint()
            if n > len(r.d):
                raise GobError("slice too long")
            vals = [self._value(t.elem, r) for _ in range(n)]
            if t.elem == T_FLOAT:
                return np.array(vals, np.float64)
            if t.elem in (T_INT, T_UINT):
                return np.array(vals, np.int64)
            return vals
        if t.kind == "map":
            n = r.uint()
            return {self._hashable(self._value(t.key, r)): self._value(t.elem, r) for _ in range(n)}
        if t.kind == "gob":
            return r.bytes()
        raise GobError(f"cannot decode {t.kind}")

    @staticmethod
    def _hashable(k):
        return k if not isinstance(k, (list, dict, np.ndarray)) else repr(k)

    def _interface(self, r: _In):
        name = r.bytes().decode()
        if not name:
            return None
        while True:  # type definitions of the concrete type, then its id
            tid = r.int()
            if tid >= 0:
                break
            self.types[-tid] = self._wire_type(r)
        sub = _In(r.take(r.uint()))
        t = self.types.get(tid)
        if t is not None and t.kind != "struct" and sub.uint() != 0:
            raise GobError("non-zero singleton delta")
        return {"type": name, "value": self._value(tid, sub)}

    def next_value(self):
        """The next top-level value, after any type definitions before it."""
        while not self.inp.done():
            msg = _In(self.inp.take(self.inp.uint()))
            tid = msg.int()
            if tid < 0:
                self.types[-tid] = self._wire_type(msg)
                continue
            t = self.types.get(tid)
            if (t is None or t.kind != "struct") and msg.uint() != 0:
                raise GobError("non-zero singleton delta")
            v = self._value(tid, msg)
            return v
        raise GobError("no value in stream")


def decode(data: bytes):
    """The first top-level value of a gob stream."""
    return Decoder(data).next_value()


# ---- save.File ----

_PARAMS = Struct("Params", [("Dt", FLOAT), ("Softening", FLOAT), ("C", FLOAT), ("DarkMatterOff", BOOL)])
_FLOATS = Slice(FLOAT)
# sim.Forces (sim.go:187-191): RestoreForces (sim.go:208-212) installs a saved evaluation only when
# AccX and Rho both hold one entry per body, so Rho is written too (zeros: no gas density here).
_FORCES = Struct("Forces", [("AccX", _FLOATS), ("AccY", _FLOATS), ("AccZ", _FLOATS), ("Rho", _FLOATS)])
_FILE = Struct("File", [
    ("Format", INT), ("Params", _PARAMS), ("Time", FLOAT), ("Steps", INT),
    ("PosX", _FLOATS), ("PosY", _FLOATS), ("PosZ", _FLOATS), ("VelX", _FLOATS), ("VelY", _FLOATS),
    ("VelZ", _FLOATS), ("Mass", _FLOATS), ("Kind", BYTES), ("Forces", _FORCES)])


def save(path: str, state: dict, params: dict, time: float = 0.0, steps: int = 0, forces=None) -> None:
    """Writes a snapshot: state holds px..vz, mass and kind (numpy arrays in state order);
    params Dt, Softening, C, DarkMatterOff; forces (ax, ay, az) of the last force evaluation or
    None (save.go:66-82 captures the same, plus fields this library does not own)."""
    f = {"Format": FORMAT, "Time": time, "Steps": steps,
         "Params": {k: params.get(k, 0) for k in ("Dt", "Softening", "C", "DarkMatterOff")},
         "PosX": state["px"], "PosY": state["py"], "PosZ": state["pz"],
         "VelX": state["vx"], "VelY": state["vy"], "VelZ": state["vz"], "Mass": state["mass"],
         "Kind": np.asarray(state.get("kind", np.zeros(len(state["mass"]), np.uint8)), np.uint8).tobytes()}
    if forces is not None:
        f["Forces"] = {"AccX": forces[0], "AccY": forces[1], "AccZ": forces[2],
                       "Rho": np.zeros(len(state["mass"]))}
    data = Encoder().encode(_FILE, f).getvalue()
    with gzip.open(path, "wb") as g:
        g.write(data)


def read(path: str) -> dict:
    """The decoded save.File of a snapshot, every field the stream holds (save.go:148-170)."""
    with open(path, "rb") as fh:
        raw = fh.read()
    try:
        data = gzip.decompress(raw)
    except (OSError, EOFError) as e:
        raise GobError(f"not a gzip stream: {e}") from e
    f = decode(data)
    if not isinstance(f, dict):
        raise GobError("the snapshot does not hold a struct")
    fmt = f.get("Format", 0)
    if not 1 <= fmt <= FORMAT:
        raise GobError(f"unsupported snapshot format {fmt}")
    return f


def load_state(path: str):
    """(state, params, meta) of a snapshot: state as the dict of arrays the library takes
    (px..vz, mass, kind, alive, and ax..az when the snapshot holds forces), params the
    sim.Params fields, meta Time, Steps and whether forces were present."""
    f = read(path)
    n = len(f.get("Mass", []))

    def arr(k):
        a = f.get(k)
        return np.zeros(n) if a is None or len(a) == 0 else np.ascontiguousarray(a, np.float64)

    kind = np.frombuffer(f.get("Kind", b""), np.uint8).copy() if f.get("Kind") else np.zeros(n, np.uint8)
    state = {"px": arr("PosX"), "py": arr("PosY"), "pz": arr("PosZ"), "vx": arr("VelX"), "vy": arr("VelY"),
             "vz": arr("VelZ"), "mass": arr("Mass"), "kind": kind, "alive": np.ones(n, np.uint8)}
    forces = f.get("Forces") or {}
    has_forces = all(len(forces.get(k, [])) == n for k in ("AccX", "AccY", "AccZ")) and n > 0
    for k, fk in (("ax", "AccX"), ("ay", "AccY"), ("az", "AccZ")):
        state[k] = np.ascontiguousarray(forces[fk], np.float64) if has_forces else np.zeros(n)
    params = dict(f.get("Params", {}))
    meta = {"Time": f.get("Time", 0.0), "Steps": f.get("Steps", 0), "Format": f.get("Format", 0),
            "forces": has_forces}
    return state, params, meta
