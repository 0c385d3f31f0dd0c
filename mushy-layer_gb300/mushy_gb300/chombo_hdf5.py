"""Minimal reader of Chombo HDF5 plot/checkpoint files, pure numpy.

Chombo writes HDF5 with superblock version 0, version-1 object headers,
symbol-table groups (v1 B-trees, SNOD nodes, local heaps) and contiguous
datasets.  This module implements exactly that subset of the published HDF5
file format so the reference's data files (e.g. plt*.2d.hdf5 written by
AMRLevelMushyLayer) can be read without h5py or libhdf5.

`read_plotfile(path)` returns the root attributes, the component names and,
per level, the boxes and the cell data per component (Fortran order inside
each box, i fastest), the layout plotting/MushyPltFile.py relies on.
`read_checkpoint(path)` reads a checkpoint's per-variable datasets, cell
(FArrayBox) and face (FluxBox) variables, as plotting/ChkFile.py does, and
`level_state` turns a one-box level into the operators' (H, C) layout.
"""
import struct

import numpy as np


class _Reader:
    def __init__(self, data):
        self.d = data
        if data[:8] != b"\x89HDF\r\n\x1a\n":
            raise ValueError("not an HDF5 file")
        sb_ver = data[8]
        if sb_ver not in (0, 1):
            raise ValueError("unsupported superblock version %d" % sb_ver)
        self.so = data[13]  # size of offsets
        self.sl = data[14]  # size of lengths
        if self.so != 8 or self.sl != 8:
            raise ValueError("only 8-byte offsets/lengths supported")
        p = 24 if sb_ver == 0 else 28
        self.base, _, self.eof, _ = struct.unpack_from("<4Q", data, p)
        p += 32
        # root group symbol table entry
        self.root = self._symbol_entry(p)

    def u(self, fmt, off):
        return struct.unpack_from("<" + fmt, self.d, off)

    def _symbol_entry(self, p):
        name_off, hdr = self.u("QQ", p)
        cache_type = self.u("I", p + 16)[0]
        scratch = self.d[p + 24:p + 40]
        btree = heap = None
        if cache_type == 1:
            btree, heap = struct.unpack_from("<QQ", scratch, 0)
        return {"name_off": name_off, "header": hdr, "btree": btree, "heap": heap}

    # ----------------------------------------------------------- objects
    def messages(self, addr):
        """Version-1 object header messages (type, flags, body bytes)."""
        d = self.d
        ver = d[addr]
        if ver != 1:
            raise ValueError("unsupported object header version %d at %d" % (ver, addr))
        nmsg = self.u("H", addr + 2)[0]
        size = self.u("I", addr + 8)[0]
        blocks = [(addr + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            p, n = blocks.pop(0)
            end = p + n
            while p + 8 <= end and len(out) < nmsg:
                mtype, msize, flags = self.u("HHB", p)
                body = d[p + 8:p + 8 + msize]
                if mtype == 0x10:  # continuation
                    coff, clen = struct.unpack_from("<QQ", body, 0)
                    blocks.append((coff, clen))
                out.append((mtype, flags, body))
                p += 8 + msize
        return out

    def local_heap_data(self, addr):
        if self.d[addr:addr + 4] != b"HEAP":
            raise ValueError("bad local heap")
        dsize, free, daddr = self.u("QQQ", addr + 8)
        return daddr

    def cstr(self, off):
        e = self.d.index(b"\x00", off)
        return self.d[off:e].decode()

    def group_entries(self, btree, heap):
        hdata = self.local_heap_data(heap)
        out = {}

        def walk(node):
            if self.d[node:node + 4] != b"TREE":
                raise ValueError("bad B-tree node")
            ntype, level, nent = self.d[node + 4], self.d[node + 5], self.u("H", node + 6)[0]
            p = node + 8 + 16  # after left/right sibling addresses
            keys_children = []
            for i in range(nent):
                p += self.sl  # key
                child = self.u("Q", p)[0]
                p += 8
                keys_children.append(child)
            for child in keys_children:
                if level > 0:
                    walk(child)
                else:
                    snod(child)

        def snod(addr):
            if self.d[addr:addr + 4] != b"SNOD":
                raise ValueError("bad symbol node")
            nsym = self.u("H", addr + 6)[0]
            p = addr + 8
            for i in range(nsym):
                e = self._symbol_entry(p)
                out[self.cstr(hdata + e["name_off"])] = e
                p += 40

        walk(btree)
        return out

    # ------------------------------------------------------ message parsing
    def dataspace(self, body):
        ver, ndim, flags = body[0], body[1], body[2]
        p = 8 if ver == 1 else 4
        dims = list(struct.unpack_from("<%dQ" % ndim, body, p))
        return dims

    def datatype(self, body):
        cv = body[0]
        cls, ver = cv & 0x0F, cv >> 4
        bits = body[1:4]
        size = struct.unpack_from("<I", body, 4)[0]
        if cls == 0:
            signed = bool(bits[0] & 0x08)
            return np.dtype(("<i%d" if signed else "<u%d") % size), 8 + 4
        if cls == 1:
            return np.dtype("<f%d" % size), 8 + 12
        if cls == 3:
            return np.dtype("S%d" % size), 8
        if cls == 6:
            nmemb = bits[0] | (bits[1] << 8)
            p = 8
            names, fmts, offs = [], [], []
            for m in range(nmemb):
                start = p
                e = body.index(b"\x00", p)
                name = body[p:e].decode()
                if ver < 3:
                    nlen = e + 1 - start
                    p = start + nlen + (-nlen) % 8  # names padded to multiple of 8
                    moff = struct.unpack_from("<I", body, p)[0]
                    p += 4 + 1 + 3 + 4 + 4 + 16  # dimensionality, reserved, perm, reserved, dims
                else:
                    p = e + 1
                    moff = int.from_bytes(body[p:p + 4], "little")
                    p += 4
                mdt, used = self.datatype(body[p:])
                p += used
                names.append(name)
                fmts.append(mdt)
                offs.append(moff)
            return np.dtype({"names": names, "formats": fmts, "offsets": offs,
                             "itemsize": size}), p
        raise ValueError("unsupported datatype class %d" % cls)

    def attributes(self, addr):
        attrs = {}
        for mtype, flags, body in self.messages(addr):
            if mtype != 0x0C:
                continue
            ver = body[0]
            nlen, dtlen, dslen = struct.unpack_from("<HHH", body, 2)
            p = 8
            name = body[p:p + nlen].split(b"\x00")[0].decode()
            pad = (lambda n: n + (-n) % 8) if ver == 1 else (lambda n: n)
            p += pad(nlen)
            dt, _ = self.datatype(body[p:p + dtlen])
            p += pad(dtlen)
            dims = self.dataspace(body[p:p + dslen])
            p += pad(dslen)
            count = int(np.prod(dims)) if dims else 1
            arr = np.frombuffer(body, dtype=dt, count=count, offset=p)
            if dt.kind == "S":
                val = arr[0].split(b"\x00")[0].decode()
            elif count == 1 and not dims:
                val = arr[0]
            else:
                val = arr.reshape(dims) if dims else arr
            attrs[name] = val
        return attrs

    def dataset(self, addr):
        dims, dt, layout = None, None, None
        for mtype, flags, body in self.messages(addr):
            if mtype == 0x01:
                dims = self.dataspace(body)
            elif mtype == 0x03:
                dt, _ = self.datatype(body)
            elif mtype == 0x08:
                layout = body
        if layout is None or dt is None:
            raise ValueError("dataset without layout/datatype")
        ver = layout[0]
        if ver == 3:
            cls = layout[1]
            if cls == 1:  # contiguous
                off, size = struct.unpack_from("<QQ", layout, 2)
                count = int(np.prod(dims)) if dims else 1
                if off == 0xFFFFFFFFFFFFFFFF:
                    return np.zeros(dims, dtype=dt)
                return np.frombuffer(self.d, dtype=dt, count=count, offset=off).reshape(dims)
            if cls == 0:  # compact
                size = struct.unpack_from("<H", layout, 2)[0]
                count = int(np.prod(dims)) if dims else 1
                return np.frombuffer(layout, dtype=dt, count=count, offset=4).reshape(dims)
            raise ValueError("chunked datasets are not supported")
        if ver in (1, 2):
            ndim = layout[1]
            cls = layout[2]
            if cls != 1:
                raise ValueError("only contiguous v1/v2 layouts supported")
            off = struct.unpack_from("<Q", layout, 8)[0]
            count = int(np.prod(dims)) if dims else 1
            return np.frombuffer(self.d, dtype=dt, count=count, offset=off).reshape(dims)
        raise ValueError("unsupported layout version %d" % ver)


def read_plotfile(path):
    data = open(path, "rb").read()
    R = _Reader(data)
    root = R.root
    attrs = R.attributes(root["header"])
    # root group's B-tree/heap come from its symbol table message
    entries = _group_children(R, root["header"])
    ncomp = int(attrs.get("num_components", 0))
    names = [attrs["component_%d" % i] for i in range(ncomp)]
    levels = []
    lev = 0
    while "level_%d" % lev in entries:
        ge = entries["level_%d" % lev]
        lattrs = R.attributes(ge["header"])
        kids = _group_children(R, ge["header"])
        boxes = R.dataset(kids["boxes"]["header"])
        offsets = R.dataset(kids["data:offsets=0"]["header"])
        flat = R.dataset(kids["data:datatype=0"]["header"])
        dattrs = R.attributes(kids["data_attributes"]["header"]) if "data_attributes" in kids else {}
        ghost = dattrs.get("outputGhost", None)
        lb = []
        for b, box in enumerate(boxes):
            f = list(box.tolist())
            dim = len(f) // 2
            lo, hi = np.array(f[:dim]), np.array(f[dim:])
            g = np.zeros(dim, dtype=int)
            if ghost is not None:
                gv = list(ghost.tolist()) if hasattr(ghost, "tolist") else [ghost]
                g = np.array(gv[:dim], dtype=int) if len(gv) >= dim else g
            ext = (hi - lo + 1) + 2 * g
            ncell = int(np.prod(ext))
            chunk = flat[int(offsets[b]):int(offsets[b]) + ncell * ncomp]
            arr = chunk.reshape((ncomp,) + tuple(ext[::-1]))
            if g.any():
                sl = (slice(None),) + tuple(slice(gg, gg + e) for gg, e in
                                           zip(g[::-1], (hi - lo + 1)[::-1]))
                arr = arr[sl]
            lb.append({"lo": lo, "hi": hi, "data": np.ascontiguousarray(arr)})
        levels.append({"attrs": lattrs, "boxes": lb})
        lev += 1
    return {"attrs": attrs, "components": names, "levels": levels}


def _extent(lo, hi):
    return np.asarray(hi) - np.asarray(lo) + 1


def _strip(arr, ghost, ext):
    """Valid region of one component block of shape ext[::-1] + 2 ghost."""
    if not np.any(ghost):
        return arr
    sl = (slice(None),) + tuple(slice(g, g + e) for g, e in zip(ghost[::-1], ext[::-1]))
    return arr[sl]


def _unpack_box(chunk, ncomp, ext, ghost):
    """One box of a checkpoint variable: a cell field (FArrayBox, comp-major,
    i fastest) or a face field (FluxBox: the faces normal to direction 0 for
    every component, then direction 1, ...), told apart by the chunk size."""
    dim = len(ext)
    ncell = int(np.prod(ext + 2 * ghost))
    if chunk.size == ncomp * ncell:
        arr = chunk.reshape((ncomp,) + tuple((ext + 2 * ghost)[::-1]))
        return np.ascontiguousarray(_strip(arr, ghost, ext))
    nface = [int(np.prod(ext + 2 * ghost + (np.arange(dim) == d))) for d in range(dim)]
    if chunk.size == ncomp * sum(nface):
        out, p = [], 0
        for d in range(dim):
            fext = ext + (np.arange(dim) == d)
            arr = chunk[p:p + ncomp * nface[d]].reshape((ncomp,) + tuple((fext + 2 * ghost)[::-1]))
            out.append(np.ascontiguousarray(_strip(arr, ghost, fext)))
            p += ncomp * nface[d]
        return out
    raise ValueError("box of %d values matches neither %d cells nor %d faces x %d components"
                     % (chunk.size, ncell, sum(nface), ncomp))


def read_checkpoint(path):
    """A Chombo checkpoint (chk*.hdf5, AMRLevelMushyLayer::writeCheckpointLevel):
    per level, one dataset per variable (`<name>:datatype=0` with its
    `<name>:offsets=0` box offsets and `<name>_attributes` {comps, ghost,
    outputGhost, objectType}) instead of the plotfile's single `data` block;
    the layout plotting/ChkFile.py:118-260 reads.

    Returns {"attrs", "space_dim", "components", "levels"}; each level holds
    its attributes, its boxes as (lo, hi) pairs and `fields`: variable name ->
    one entry per box, an array (comps, [nz,] ny, nx) for cell variables or a
    list of D arrays (comps, face extents) for face variables such as the
    advection velocity `advVel`."""
    data = open(path, "rb").read()
    R = _Reader(data)
    attrs = R.attributes(R.root["header"])
    entries = _group_children(R, R.root["header"])
    glob = R.attributes(entries["Chombo_global"]["header"]) if "Chombo_global" in entries else {}
    ncomp = int(attrs.get("num_components", 0))
    levels = []
    lev = 0
    while "level_%d" % lev in entries:
        ge = entries["level_%d" % lev]
        lattrs = R.attributes(ge["header"])
        kids = _group_children(R, ge["header"])
        raw = R.dataset(kids["boxes"]["header"])
        boxes = []
        for box in raw:
            f = list(box.tolist())
            dim = len(f) // 2
            boxes.append((np.array(f[:dim]), np.array(f[dim:])))
        fields = {}
        for key in sorted(kids):
            if not key.endswith(":datatype=0"):
                continue
            name = key[:-len(":datatype=0")]
            va = R.attributes(kids[name + "_attributes"]["header"]) \
                if name + "_attributes" in kids else {}
            nc = int(va.get("comps", 1))
            ghost = va.get("outputGhost", None)
            flat = R.dataset(kids[key]["header"])
            offs = R.dataset(kids[name + ":offsets=0"]["header"])
            per_box = []
            for b, (lo, hi) in enumerate(boxes):
                g = np.zeros(len(lo), dtype=int)
                if ghost is not None:
                    gv = list(ghost.tolist()) if hasattr(ghost, "tolist") else [ghost]
                    g = np.array(gv[:len(lo)], dtype=int)
                chunk = flat[int(offs[b]):int(offs[b + 1])]
                per_box.append(_unpack_box(chunk, nc, _extent(lo, hi), g))
            fields[name] = per_box
        levels.append({"attrs": lattrs, "boxes": boxes, "fields": fields})
        lev += 1
    return {"attrs": attrs, "space_dim": int(glob.get("SpaceDim", len(levels[0]["boxes"][0][0])
                                                      if levels else 0)),
            "components": [attrs["component_%d" % i] for i in range(ncomp)],
            "levels": levels}


def level_state(chk, level, names=("Enthalpy", "Bulk concentration")):
    """The (H, C) state of a one-box checkpoint level in the layout of the
    operators, [comp][k][j][i] (k of extent 1 in 2D), with the level's box
    and spacing: a restart state for NLMultiCompOp / the solvers."""
    L = chk["levels"][level]
    if len(L["boxes"]) != 1:
        raise ValueError("level %d has %d boxes; one box per level is needed"
                         % (level, len(L["boxes"])))
    comps = []
    for name in names:
        a = L["fields"][name][0]
        if isinstance(a, list):
            raise ValueError("%s is a face variable" % name)
        comps.extend(a)
    st = np.stack(comps)
    if st.ndim == 3:
        st = st[:, None]
    lo, hi = L["boxes"][0]
    return np.ascontiguousarray(st), (lo, hi), float(L["attrs"]["dx"])


def _group_children(R, header):
    for mtype, flags, body in R.messages(header):
        if mtype == 0x11:
            btree, heap = struct.unpack_from("<QQ", body, 0)
            return R.group_entries(btree, heap)
    return {}
