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

Covered, for reading and for writing back byte for byte: NULL and R's singleton environments,
symbols, dotted pairs (pairlists, calls, closures, promises), environments (and package / namespace
environments by name), primitives, external pointers and weak references, logical / integer /
double / complex / character / list / expression / raw vectors, S4 objects, attributes, ALTREP
items and compiled byte code (kept as the grammar it was read in), in formats 2 and 3.
"""
import gzip
import struct

import numpy as np

NILSXP, SYMSXP, LISTSXP, CLOSXP, ENVSXP, PROMSXP, LANGSXP, SPECIALSXP, BUILTINSXP, CHARSXP = 0, 1, 2, 3, 4, 5, 6, 7, 8, 9
LGLSXP, INTSXP, REALSXP, CPLXSXP, STRSXP, DOTSXP, VECSXP, EXPRSXP, BCODESXP = 10, 13, 14, 15, 16, 17, 19, 20, 21
EXTPTRSXP, WEAKREFSXP, RAWSXP, S4SXP = 22, 23, 24, 25
ALTREP_SXP, ATTRLISTSXP, ATTRLANGSXP, BCREPREF, BCREPDEF = 238, 239, 240, 243, 244
PACKAGESXP, NAMESPACESXP, REFSXP, NILVALUE_SXP = 248, 249, 255, 254
# singleton environments and markers, written as their code alone
_SPECIAL = {253: "globalenv", 252: "unbound", 251: "missingarg", 250: "basenamespace", 242: "emptyenv",
            241: "baseenv"}
# dotted-pair types: (attributes), (tag), car, then the cdr as the next item
_PAIRS = (LISTSXP, LANGSXP, CLOSXP, PROMSXP, DOTSXP)
NA_INTEGER = -2 ** 31
NA_LOGICAL = NA_INTEGER
_IS_OBJECT, _HAS_ATTR, _HAS_TAG = 1 << 8, 1 << 9, 1 << 10
_ASCII_MASK, _UTF8_MASK, _LATIN1_MASK, _BYTES_MASK = 1 << 6, 1 << 3, 1 << 2, 1 << 1
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


class RChar(str):
    """A string whose encoding bits differ from the ones this writer derives (ASCII, else UTF-8)."""

    def __new__(cls, value, levels):
        obj = str.__new__(cls, value)
        obj.levels = levels
        return obj


class RObj:
    """An R vector or dotted pair: ``type`` (SEXPTYPE), ``value`` and ``attrs`` (a list of (name, value)
    pairs in the order R keeps them).

    value by type: logical / integer -> int32 array (NA = -2^31), double -> float64 array, complex ->
    complex128 array, character -> list of str (None = NA), list / expression -> list of items, raw ->
    bytes.  Dotted pairs (pairlist, call, closure, promise, ...) -> list of (tag, car), the tag a
    symbol's name, None, or another item (a closure's environment); ``tail`` is the last node's cdr
    when it is not NULL.  A pairlist keeps its nodes in one list; the other dotted-pair types hold
    one node and their cdr in ``tail``.  ``levels`` are the item's general-purpose bits as read."""
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


class REnv:
    """An environment: locked flag, enclosure, frame (a pairlist), hash table (a list), attributes.
    Referred to by identity: the items that point at it share this object."""
    __slots__ = ("locked", "enclos", "frame", "hashtab", "attrib")

    def __init__(self, locked=0, enclos=None, frame=None, hashtab=None, attrib=None):
        self.locked, self.enclos, self.frame, self.hashtab, self.attrib = locked, enclos, frame, hashtab, attrib


class RNamedEnv:
    """A package or namespace environment, written as its name strings (type PACKAGESXP or
    NAMESPACESXP) and found again by name when R loads it."""
    __slots__ = ("type", "names")

    def __init__(self, type_, names):
        self.type, self.names = type_, list(names)


class RPrim:
    """A primitive function (SPECIALSXP / BUILTINSXP), written as its name."""
    __slots__ = ("type", "name", "attrs", "levels", "is_object")

    def __init__(self, type_, name, attrs=None, levels=0, is_object=False):
        self.type, self.name, self.attrs, self.levels, self.is_object = type_, name, list(attrs or []), levels, is_object


class RExtPtr:
    """An external pointer (its address is not serialised): protected value, tag, attributes."""
    __slots__ = ("prot", "tag", "attrs", "levels", "is_object")

    def __init__(self, prot, tag, attrs=None, levels=0, is_object=False):
        self.prot, self.tag, self.attrs, self.levels, self.is_object = prot, tag, list(attrs or []), levels, is_object


class RWeakRef:
    """A weak reference (serialised empty)."""
    __slots__ = ("attrs", "levels", "is_object")

    def __init__(self, attrs=None, levels=0, is_object=False):
        self.attrs, self.levels, self.is_object = list(attrs or []), levels, is_object


class RBytecode:
    """Compiled code as serialised: the number of shared cells (``nreps``) and the code, a tree of
    (code item, constants).  A constant is ("bc", code), ("lang", node) or ("item", type, item); a
    language node is ("ref", index), ("node", def index or None, type, attrs, tag, car, cdr) with car
    and cdr again nodes, or ("leaf", item)."""
    __slots__ = ("nreps", "code", "attrs", "levels", "is_object")

    def __init__(self, nreps, code, attrs=None, levels=0, is_object=False):
        self.nreps, self.code, self.attrs, self.levels, self.is_object = nreps, code, list(attrs or []), levels, is_object


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
        raw = bytes(self.b[self.o:self.o + n])
        self.o += n
        levels = (flags >> 12) & (_ASCII_MASK | _UTF8_MASK | _LATIN1_MASK | _BYTES_MASK)
        s = raw.decode("latin-1" if levels & (_LATIN1_MASK | _BYTES_MASK) else "utf-8")
        derived = _ASCII_MASK if all(c < 128 for c in raw) else _UTF8_MASK
        return s if levels == derived and not levels & _BYTES_MASK else RChar(s, flags >> 12)

    def attrs_of(self, has_attr):
        if not has_attr:
            return []
        pl = self.item()
        if not (isinstance(pl, RObj) and pl.type == LISTSXP):
            raise ValueError("attributes are not a pairlist")
        return [(k, v) for k, v in pl.value]

    def strvec(self):
        if self.int() != 0:
            raise ValueError("names of a string vector are not supported")
        return [self.item() for _ in range(self.int())]

    def tag_of(self, has_tag):
        if not has_tag:
            return None
        t = self.item()
        return t.name if isinstance(t, RSym) else t

    def bc_lang(self, kind):
        if kind == BCREPREF:
            return ("ref", self.int())
        if kind in (BCREPDEF, LANGSXP, LISTSXP, ATTRLANGSXP, ATTRLISTSXP):
            pos = None
            if kind == BCREPDEF:
                pos = self.int()
                kind = self.int()
            attrs = self.item() if kind in (ATTRLANGSXP, ATTRLISTSXP) else None
            tag = self.item()
            car = self.bc_lang(self.int())
            cdr = self.bc_lang(self.int())
            return ("node", pos, kind, attrs, tag, car, cdr)
        return ("leaf", self.item())

    def bc1(self):
        code = self.item()
        consts = []
        for _ in range(self.int()):
            kind = self.int()
            if kind == BCODESXP:
                consts.append(("bc", self.bc1()))
            elif kind in (LANGSXP, LISTSXP, BCREPDEF, BCREPREF, ATTRLANGSXP, ATTRLISTSXP):
                consts.append(("lang", self.bc_lang(kind)))
            else:
                consts.append(("item", kind, self.item()))
        return (code, consts)

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
        if t in (PACKAGESXP, NAMESPACESXP):
            env = RNamedEnv(t, self.strvec())
            self.refs.append(env)
            return env
        if t == ENVSXP:
            env = REnv()
            self.refs.append(env)  # before its contents, which may refer to it
            env.locked = self.int()
            env.enclos, env.frame, env.hashtab, env.attrib = self.item(), self.item(), self.item(), self.item()
            return env
        if t in _PAIRS:
            # one node, or for a pairlist every plain node of the chain; a cdr of another kind (or a
            # pairlist node with attributes, an object bit or other bits) is the tail item
            items = []
            node_attrs = self.attrs_of(has_attr)
            tail = None
            while True:
                tag = self.tag_of(has_tag)
                items.append((tag, self.item()))
                nflags = self.int()
                if nflags == NILVALUE_SXP:
                    break
                if t == LISTSXP and nflags in (LISTSXP, LISTSXP | _HAS_TAG):
                    has_tag = bool(nflags & _HAS_TAG)
                    continue
                self.o -= 4
                tail = self.item()
                break
            return RObj(t, items, node_attrs, levels, is_obj, tail)
        if t == ALTREP_SXP:
            info = self.item()
            state = self.item()
            attr = self.item()
            return RAltrep(info, state, attr, flags)
        if t == CHARSXP:
            return self.charsxp(flags)
        if t in (SPECIALSXP, BUILTINSXP):
            n = self.int()
            name = bytes(self.b[self.o:self.o + n]).decode("latin-1")
            self.o += n
            return RPrim(t, name, self.attrs_of(has_attr), levels, is_obj)
        if t == EXTPTRSXP:
            x = RExtPtr(None, None, None, levels, is_obj)
            self.refs.append(x)
            x.prot, x.tag = self.item(), self.item()
            x.attrs = self.attrs_of(has_attr)
            return x
        if t == WEAKREFSXP:
            x = RWeakRef(None, levels, is_obj)
            self.refs.append(x)
            x.attrs = self.attrs_of(has_attr)
            return x
        if t == BCODESXP:
            nreps = self.int()
            code = self.bc1()
            return RBytecode(nreps, code, self.attrs_of(has_attr), levels, is_obj)
        if t == S4SXP:
            return RObj(t, None, self.attrs_of(has_attr), levels, is_obj)
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
    def __init__(self, version=3):
        self.parts = []
        self.refs = {}
        self.version = version

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
        raw = s.encode("latin-1") if isinstance(s, RChar) and s.levels & (_LATIN1_MASK | _BYTES_MASK) \
            else s.encode("utf-8")
        if isinstance(s, RChar):
            levels = s.levels
        else:
            levels = _ASCII_MASK if all(c < 128 for c in raw) else _UTF8_MASK
        self.int(CHARSXP | (levels << 12))
        self.int(len(raw))
        self.parts.append(raw)

    def attrs(self, attrs):
        if attrs:
            self.item(RObj(LISTSXP, list(attrs)))

    def flags(self, t, levels, is_object, has_attr, has_tag=False):
        self.int(t | (levels << 12) | (_IS_OBJECT if is_object else 0) | (_HAS_ATTR if has_attr else 0)
                 | (_HAS_TAG if has_tag else 0))

    def tag(self, tag):
        self.item(RSym(tag) if isinstance(tag, str) else tag)

    def bc_lang(self, node):
        kind = node[0]
        if kind == "ref":
            self.int(BCREPREF)
            self.int(node[1])
        elif kind == "node":
            _, pos, t, attrs, tag, car, cdr = node
            if pos is not None:
                self.int(BCREPDEF)
                self.int(pos)
            self.int(t)
            if t in (ATTRLANGSXP, ATTRLISTSXP):
                self.item(attrs)
            self.item(tag)
            self.bc_lang(car)
            self.bc_lang(cdr)
        else:
            self.int(0)
            self.item(node[1])

    def bc1(self, code):
        body, consts = code
        self.item(body)
        self.int(len(consts))
        for c in consts:
            if c[0] == "bc":
                self.int(BCODESXP)
                self.bc1(c[1])
            elif c[0] == "lang":
                self.bc_lang(c[1])  # writes its own type word
            else:
                self.int(c[1])
                self.item(c[2])

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
        if isinstance(x, (REnv, RNamedEnv, RExtPtr, RWeakRef)):
            if self.ref_or_add(("id", id(x))):
                return
            if isinstance(x, RNamedEnv):
                self.int(x.type)
                self.int(0)
                self.int(len(x.names))
                for s in x.names:
                    self.item(s)
            elif isinstance(x, REnv):
                self.int(ENVSXP)
                self.int(x.locked)
                for part in (x.enclos, x.frame, x.hashtab, x.attrib):
                    self.item(part)
            elif isinstance(x, RExtPtr):
                self.flags(EXTPTRSXP, x.levels, x.is_object, bool(x.attrs))
                self.item(x.prot)
                self.item(x.tag)
                self.attrs(x.attrs)
            else:
                self.flags(WEAKREFSXP, x.levels, x.is_object, bool(x.attrs))
                self.attrs(x.attrs)
            return
        if isinstance(x, str):  # a CHARSXP item (a namespace's name strings)
            self.charsxp(x)
            return
        if isinstance(x, RAltrep):
            self.int(x.flags)
            self.item(x.info)
            self.item(x.state)
            self.item(x.attrs)
            return
        if isinstance(x, RPrim):
            self.flags(x.type, x.levels, x.is_object, bool(x.attrs))
            raw = x.name.encode("latin-1")
            self.int(len(raw))
            self.parts.append(raw)
            self.attrs(x.attrs)
            return
        if isinstance(x, RBytecode):
            self.flags(BCODESXP, x.levels, x.is_object, bool(x.attrs))
            self.int(x.nreps)
            self.bc1(x.code)
            self.attrs(x.attrs)
            return
        if not isinstance(x, RObj):
            raise TypeError("cannot serialise %r" % type(x))
        t = x.type
        if t in _PAIRS:
            # the first node carries the item's levels, object bit and attributes; a pairlist's
            # further nodes are plain
            first = True
            for tag, car in x.value:
                if first:
                    self.flags(t, x.levels, x.is_object, bool(x.attrs), tag is not None)
                    self.attrs(x.attrs)
                else:
                    self.flags(LISTSXP, 0, False, False, tag is not None)
                if tag is not None:
                    self.tag(tag)
                self.item(car)
                first = False
            if x.tail is None:
                self.int(NILVALUE_SXP)
            else:
                self.item(x.tail)
            return
        self.flags(t, x.levels, x.is_object, bool(x.attrs))
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
        elif t == S4SXP:
            pass
        else:
            raise NotImplementedError("R item type %d is not supported" % t)
        self.attrs(x.attrs)


def serialize(obj, writer=R_VERSION_4_3_2, min_reader=None, encoding="UTF-8", version=3):
    """XDR serialisation of one item, format 3 (with the native encoding) or 2.  The reader's
    header dict may be passed back as keyword arguments."""
    if version not in (2, 3):
        raise ValueError("serialisation format %r" % version)
    w = _Writer()
    w.parts.append(b"X\n")
    w.int(version)
    w.int(writer)
    if min_reader is None:  # the oldest R that reads the format: 3.5.0 for format 3, 2.3.0 for 2
        min_reader = R_VERSION_3_5_0 if version == 3 else (2 << 16) | (3 << 8)
    w.int(min_reader)
    if version == 3:
        w.int(len(encoding))
        w.parts.append(encoding.encode("ascii"))
    w.item(obj)
    return b"".join(w.parts)


def rda_bytes(objects, **header):
    """The uncompressed bytes save() writes for [(name, object)]."""
    magic = b"RDX2\n" if header.get("version", 3) == 2 else b"RDX3\n"
    return magic + serialize(RObj(LISTSXP, list(objects)), **header)


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
