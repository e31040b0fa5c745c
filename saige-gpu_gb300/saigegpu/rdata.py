"""R's XDR serialisation, format version 3: the .rda files the reference's step 1 writes with save()
(FIT.R:1218, 1299) and its step 2 reads with load().

The format is R's own (R Internals, "Serialization Formats"): an "RDX3\\n" magic for save() files, then
"X\\n", three integers (format version 3, the writing R's version, the oldest R that reads it), the
native encoding, and one item: a pairlist whose tags are the saved objects' names.  An item is a
32-bit flags word (type in the low byte, the object bit 1 << 8, has-attributes 1 << 9, has-tag
1 << 10, the general-purpose "levels" bits above 1 << 12) followed by its data: big-endian integers
and IEEE doubles, lengths as 32-bit integers (-1 then two words for long vectors), strings as CHARSXP
items (length, bytes; -1 for NA), attributes as a trailing pairlist.  Symbols are written once and
then referred to by their position in a table of symbols and environments (REFSXP, index << 8).

Covered: NULL, symbols, pairlists, logical / integer / double / complex / character / list /
expression / raw vectors, attributes, and ALTREP items (kept as they were read, so a file read here
writes back byte for byte); closures, environments, language objects and byte code are not (step 1's
model holds none of them except inside objects the reference rebuilds on load).
"""
import gzip
import struct

import numpy as np

NILSXP, SYMSXP, LISTSXP, CHARSXP, LGLSXP, INTSXP, REALSXP, CPLXSXP, STRSXP, VECSXP, EXPRSXP, RAWSXP = (
    0, 1, 2, 9, 10, 13, 14, 15, 16, 19, 20, 24)
ALTREP_SXP, REFSXP, NILVALUE_SXP = 238, 255, 254
_SPECIAL = {253: "globalenv", 252: "unbound", 251: "missingarg", 250: "basenamespace", 242: "emptyenv",
            241: "baseenv"}
NA_INTEGER = -2 ** 31
NA_LOGICAL = NA_INTEGER
_IS_OBJECT, _HAS_ATTR, _HAS_TAG = 1 << 8, 1 << 9, 1 << 10
_ASCII_MASK, _UTF8_MASK = 1 << 6, 1 << 3
R_VERSION_4_3_2 = (4 << 16) | (3 << 8) | 2
R_VERSION_3_5_0 = (3 << 16) | (5 << 8) | 0


class RSym:
    """An R symbol (a name)."""
    __slots__ = ("name",)

    def __init__(self, name):
        self.name = name

    def __eq__(self, other):
        return isinstance(other, RSym) and other.name == self.name

    def __hash__(self):
        return hash(("RSym", self.name))

    def __repr__(self):
        return "RSym(%r)" % self.name


class RObj:
    """An R vector or pairlist: ``type`` (SEXPTYPE), ``value`` and ``attrs`` (a list of (name, value)
    pairs in the order R keeps them).

    value by type: logical / integer -> int32 array (NA = -2^31), double -> float64 array, complex ->
    complex128 array, character -> list of str (None = NA), list / expression -> list of items, raw ->
    bytes, pairlist -> list of (tag name or None, item), with ``tail`` the last node's cdr when it
    is not NULL (a dotted pair).  ``levels`` are the item's general-purpose bits as read (0 for
    vectors R builds)."""
    __slots__ = ("type", "value", "attrs", "levels", "is_object", "tail")

    def __init__(self, type_, value, attrs=None, levels=0, is_object=None, tail=None):
        self.type = type_
        self.value = value
        self.attrs = list(attrs or [])
        self.levels = levels
        self.tail = tail
        # R sets the object bit on every item with a class attribute
        self.is_object = any(k == "class" for k, _ in self.attrs) if is_object is None else bool(is_object)

    def attr(self, name, default=None):
        for k, v in self.attrs:
            if k == name:
                return v
        return default

    def names(self):
        n = self.attr("names")
        return None if n is None else list(n.value)

    def __getitem__(self, key):
        """A list's element by name (R's ``x$name``)."""
        if self.type not in (VECSXP, EXPRSXP):
            raise TypeError("not a list")
        names = self.names() or []
        for k, v in zip(names, self.value):
            if k == key:
                return v
        raise KeyError(key)

    def __repr__(self):
        n = len(self.value) if hasattr(self.value, "__len__") else 0
        return "RObj(type=%d, len=%d, attrs=%s)" % (self.type, n, [k for k, _ in self.attrs])


class RAltrep:
    """An ALTREP item as serialised (class info, state, attributes), kept verbatim."""
    __slots__ = ("info", "state", "attrs", "flags")

    def __init__(self, info, state, attrs, flags):
        self.info, self.state, self.attrs, self.flags = info, state, attrs, flags


class RSpecial:
    """One of R's singleton environments or markers (global / base / empty environment, ...)."""
    __slots__ = ("code",)

    def __init__(self, code):
        self.code = code

    def __eq__(self, other):
        return isinstance(other, RSpecial) and other.code == self.code

    def __hash__(self):
        return hash(("RSpecial", self.code))


# ---------------------------------------------------------------------------------- reading
class _Reader:
    def __init__(self, data):
        self.b = data
        self.o = 0
        self.refs = []

    def int(self):
        v = struct.unpack_from(">i", self.b, self.o)[0]
        self.o += 4
        return v

    def length(self):
        n = self.int()
        if n == -1:
            hi, lo = self.int(), self.int()
            n = (hi << 32) + (lo & 0xFFFFFFFF)
        return n

    def charsxp(self, flags):
        n = self.int()
        if n == -1:
            return None
        raw = self.b[self.o:self.o + n]
        self.o += n
        levels = flags >> 12
        return raw.decode("latin-1" if levels & (1 << 2) else "utf-8")

    def attrs_of(self, has_attr):
        if not has_attr:
            return []
        pl = self.item()
        if not (isinstance(pl, RObj) and pl.type == LISTSXP):
            raise ValueError("attributes are not a pairlist")
        return [(k, v) for k, v in pl.value]

    def item(self):
        flags = self.int()
        t = flags & 0xFF
        levels = flags >> 12
        is_obj = bool(flags & _IS_OBJECT)
        has_attr = bool(flags & _HAS_ATTR)
        has_tag = bool(flags & _HAS_TAG)
        if t == NILVALUE_SXP:
            return None
        if t in _SPECIAL:
            return RSpecial(t)
        if t == REFSXP:
            idx = flags >> 8
            if idx == 0:
                idx = self.int()
            return self.refs[idx - 1]
        if t == SYMSXP:
            cflags = self.int()
            sym = RSym(self.charsxp(cflags))
            self.refs.append(sym)
            return sym
        if t == LISTSXP:
            # a pairlist: each node carries (attributes), (tag), car, then the next node or NULL
            items, node_attrs, tail = [], None, None
            while True:
                a = self.attrs_of(has_attr)
                if node_attrs is None:
                    node_attrs = a
                elif a:
                    raise NotImplementedError("attributes on a pairlist node after the first")
                tag = self.item() if has_tag else None
                car = self.item()
                items.append((tag.name if isinstance(tag, RSym) else None, car))
                nflags = self.int()
                nt = nflags & 0xFF
                if nt == NILVALUE_SXP:
                    break
                if nt != LISTSXP or nflags >> 12:
                    self.o -= 4
                    tail = self.item()  # a dotted pair's cdr
                    break
                has_attr = bool(nflags & _HAS_ATTR)
                has_tag = bool(nflags & _HAS_TAG)
            return RObj(LISTSXP, items, node_attrs, levels, is_obj, tail)
        if t == ALTREP_SXP:
            info = self.item()
            state = self.item()
            attr = self.item()
            return RAltrep(info, state, attr, flags)
        if t == CHARSXP:
            return self.charsxp(flags)
        if t in (LGLSXP, INTSXP):
            n = self.length()
            v = np.frombuffer(self.b, dtype=">i4", count=n, offset=self.o).astype(np.int32)
            self.o += 4 * n
        elif t == REALSXP:
            n = self.length()
            v = np.frombuffer(self.b, dtype=">f8", count=n, offset=self.o).astype(np.float64)
            self.o += 8 * n
        elif t == CPLXSXP:
            n = self.length()
            w = np.frombuffer(self.b, dtype=">f8", count=2 * n, offset=self.o).astype(np.float64)
            v = w[0::2] + 1j * w[1::2]
            self.o += 16 * n
        elif t == STRSXP:
            n = self.length()
            v = []
            for _ in range(n):
                v.append(self.charsxp(self.int()))
        elif t in (VECSXP, EXPRSXP):
            n = self.length()
            v = [self.item() for _ in range(n)]
        elif t == RAWSXP:
            n = self.length()
            v = bytes(self.b[self.o:self.o + n])
            self.o += n
        else:
            raise NotImplementedError("R item type %d is not supported" % t)
        return RObj(t, v, self.attrs_of(has_attr), levels, is_obj)


def unserialize(data):
    """(header, item) of an R serialisation stream in XDR format ('X\\n' first)."""
    r = _Reader(data)
    if data[:2] != b"X\n":
        raise ValueError("not an XDR serialisation")
    r.o = 2
    version = r.int()
    writer, min_reader = r.int(), r.int()
    header = {"version": version, "writer": writer, "min_reader": min_reader}
    if version == 3:
        n = r.int()
        header["encoding"] = r.b[r.o:r.o + n].decode("ascii")
        r.o += n
    elif version != 2:
        raise ValueError("serialisation format %d" % version)
    obj = r.item()
    if r.o != len(data):
        raise ValueError("%d bytes after the serialised item" % (len(data) - r.o))
    return header, obj


def read_rda(path):
    """(header, [(name, object)]) of a save() file (gzip'd or not)."""
    raw = open(path, "rb").read()
    if raw[:2] == b"\x1f\x8b":
        raw = gzip.decompress(raw)
    if raw[:5] not in (b"RDX2\n", b"RDX3\n"):
        raise ValueError("not an .rda file (magic %r)" % raw[:5])
    header, top = unserialize(raw[5:])
    if not (isinstance(top, RObj) and top.type == LISTSXP):
        raise ValueError("an .rda file holds a pairlist of named objects")
    return header, list(top.value)


# ---------------------------------------------------------------------------------- writing
class _Writer:
    def __init__(self):
        self.parts = []
        self.refs = {}

    def int(self, v):
        self.parts.append(struct.pack(">i", v))

    def length(self, n):
        if n > 2 ** 31 - 1:
            self.int(-1)
            self.int(n >> 32)
            self.int(n & 0xFFFFFFFF)
        else:
            self.int(n)

    def ref_or_add(self, key):
        """True (and the reference written) when key was written before; else it joins the table."""
        idx = self.refs.get(key)
        if idx is not None:
            if idx > (2 ** 31 - 1) >> 8:
                self.int(REFSXP)
                self.int(idx)
            else:
                self.int((idx << 8) | REFSXP)
            return True
        self.refs[key] = len(self.refs) + 1
        return False

    def charsxp(self, s):
        if s is None:
            self.int(CHARSXP)
            self.int(-1)
            return
        raw = s.encode("utf-8")
        levels = _ASCII_MASK if all(c < 128 for c in raw) else _UTF8_MASK
        self.int(CHARSXP | (levels << 12))
        self.int(len(raw))
        self.parts.append(raw)

    def attrs(self, attrs):
        if attrs:
            self.item(RObj(LISTSXP, list(attrs)))

    def item(self, x):
        if x is None:
            self.int(NILVALUE_SXP)
            return
        if isinstance(x, RSpecial):
            self.int(x.code)
            return
        if isinstance(x, RSym):
            if not self.ref_or_add(x):
                self.int(SYMSXP)
                self.charsxp(x.name)
            return
        if isinstance(x, RAltrep):
            self.int(x.flags)
            self.item(x.info)
            self.item(x.state)
            self.item(x.attrs)
            return
        if not isinstance(x, RObj):
            raise TypeError("cannot serialise %r" % type(x))
        t = x.type
        flags = t | (x.levels << 12) | (_IS_OBJECT if x.is_object else 0) | (_HAS_ATTR if x.attrs else 0)
        if t == LISTSXP:
            # every node after the first carries no attributes; tags are symbols
            first = True
            for tag, car in x.value:
                f = LISTSXP | (x.levels << 12 if first else 0) | (_HAS_TAG if tag is not None else 0)
                if first:
                    f |= (_IS_OBJECT if x.is_object else 0) | (_HAS_ATTR if x.attrs else 0)
                self.int(f)
                if first:
                    self.attrs(x.attrs)
                if tag is not None:
                    self.item(RSym(tag))
                self.item(car)
                first = False
            if x.tail is None:
                self.int(NILVALUE_SXP)
            else:
                self.item(x.tail)
            return
        self.int(flags)
        v = x.value
        if t in (LGLSXP, INTSXP):
            a = np.asarray(v, dtype=">i4")
            self.length(a.size)
            self.parts.append(a.tobytes())
        elif t == REALSXP:
            a = np.asarray(v, dtype=">f8")
            self.length(a.size)
            self.parts.append(a.tobytes())
        elif t == CPLXSXP:
            a = np.asarray(v, dtype=np.complex128)
            w = np.empty(2 * a.size, dtype=">f8")
            w[0::2], w[1::2] = a.real, a.imag
            self.length(a.size)
            self.parts.append(w.tobytes())
        elif t == STRSXP:
            self.length(len(v))
            for s in v:
                self.charsxp(s)
        elif t in (VECSXP, EXPRSXP):
            self.length(len(v))
            for e in v:
                self.item(e)
        elif t == RAWSXP:
            self.length(len(v))
            self.parts.append(bytes(v))
        else:
            raise NotImplementedError("R item type %d is not supported" % t)
        self.attrs(x.attrs)


def serialize(obj, writer=R_VERSION_4_3_2, min_reader=R_VERSION_3_5_0, encoding="UTF-8"):
    """XDR serialisation (format 3) of one item."""
    w = _Writer()
    w.parts.append(b"X\n")
    w.int(3)
    w.int(writer)
    w.int(min_reader)
    w.int(len(encoding))
    w.parts.append(encoding.encode("ascii"))
    w.item(obj)
    return b"".join(w.parts)


def rda_bytes(objects, **header):
    """The uncompressed bytes save() writes for [(name, object)]."""
    return b"RDX3\n" + serialize(RObj(LISTSXP, list(objects)), **header)


def write_rda(path, objects, compresslevel=6, **header):
    """save(list = names, file = path): gzip'd, as R's default."""
    with gzip.open(path, "wb", compresslevel=compresslevel) as f:
        f.write(rda_bytes(objects, **header))


# ---------------------------------------------------------------------------------- building
def r_double(x, dim=None, names=None):
    a = np.asarray(x, np.float64).ravel(order="F")
    attrs = []
    if dim is not None:
        attrs.append(("dim", r_int(list(dim))))
    if names is not None:
        attrs.append(("names", r_str(list(names))))
    return RObj(REALSXP, a, attrs)


def r_matrix(m, colnames=None):
    """A double matrix (column-major, as R holds it); colnames as dimnames = list(NULL, colnames)."""
    a = np.asarray(m, np.float64)
    if a.ndim == 1:
        a = a[:, None]
    attrs = [("dim", r_int(list(a.shape)))]
    if colnames is not None:
        attrs.append(("dimnames", r_list([None, r_str(list(colnames))])))
    return RObj(REALSXP, a.ravel(order="F"), attrs)


def r_int(x):
    return RObj(INTSXP, np.asarray(x, np.int32).ravel())


def r_lgl(x):
    a = np.atleast_1d(np.asarray(x))
    return RObj(LGLSXP, np.where(a.astype(bool), 1, 0).astype(np.int32))


def r_str(x):
    if isinstance(x, str):
        x = [x]
    return RObj(STRSXP, [None if s is None else str(s) for s in x])


def r_list(values, names=None, cls=None):
    attrs = []
    if names is not None:
        attrs.append(("names", r_str(list(names))))
    if cls is not None:
        attrs.append(("class", r_str(cls)))
    return RObj(VECSXP, list(values), attrs)


def r_named_list(pairs, cls=None):
    pairs = list(pairs)
    return r_list([v for _, v in pairs], [k for k, _ in pairs], cls)


def to_numpy(x):
    """A numeric vector or matrix as a numpy array (matrices in their R shape)."""
    if not (isinstance(x, RObj) and x.type in (LGLSXP, INTSXP, REALSXP)):
        raise TypeError("not a numeric vector")
    dim = x.attr("dim")
    a = np.asarray(x.value)
    if x.type == LGLSXP:
        a = a.astype(bool)
    if dim is not None:
        a = a.reshape(tuple(int(d) for d in dim.value), order="F")
    return a


def schema(x):
    """The structure of an item, for comparing two files' layouts: type, length, attribute names in
    order, dim, class, and the same for a list's elements ("fields", with their names) and for the
    dimnames' two parts.  ALTREP items show as "altrep"."""
    if x is None:
        return None
    if isinstance(x, RAltrep):
        return "altrep"
    if isinstance(x, RSym):
        return "symbol"
    if not isinstance(x, RObj):
        return type(x).__name__
    n = len(x.value) if hasattr(x.value, "__len__") else 0
    out = {"type": x.type, "len": n, "attrs": [k for k, _ in x.attrs]}
    dim = x.attr("dim")
    if isinstance(dim, RObj):
        out["dim"] = [int(d) for d in dim.value]
    cls = x.attr("class")
    if isinstance(cls, RObj):
        out["class"] = list(cls.value)
    dn = x.attr("dimnames")
    if isinstance(dn, RObj):
        out["dimnames"] = [schema(e) for e in dn.value]
    if x.type in (VECSXP, EXPRSXP):
        names = x.names() or [None] * n
        out["fields"] = [[k, schema(e)] for k, e in zip(names, x.value)]
    return out
