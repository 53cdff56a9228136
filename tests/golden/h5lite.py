"""Minimal pure-Python reader for the HDF5 files the reference's tests load.

The reference stores Epetra vectors with EpetraExt::HDF5 (see
src/utils/Utils.H, ``Utils::load``): one group per vector with a dataset
``Values`` (FP64) and integer attributes. h5py is not installed here, so
this module reads just that subset of the HDF5 format (file format
specification 1.8/1.10, "version 0" superblock):

- superblock version 0 or 1 with 8-byte offsets and lengths;
- version-1 object headers, with continuation blocks;
- old-style groups (symbol-table message -> group B-tree -> symbol nodes,
  names in the local heap);
- datasets of IEEE floating-point or integer type, contiguous or chunked
  storage (chunk B-tree, optional deflate filter).

``read(path)`` returns ``{"Group/Dataset": numpy.ndarray}`` for every dataset.
It is used only by the fixture scripts of tests/golden/.
"""
import struct
import zlib

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"


class _File:
    def __init__(self, data):
        self.d = data
        if data[:8] != _SIG:
            raise ValueError("not an HDF5 file")
        ver = data[8]
        if ver not in (0, 1):
            raise ValueError("superblock version %d not supported" % ver)
        self.so, self.sl = data[13], data[14]
        if self.so != 8 or self.sl != 8:
            raise ValueError("only 8-byte offsets/lengths are supported")
        pos = 24 + (4 if ver == 1 else 0)
        self.base = self.u64(pos)
        pos += 32                       # base, free-space, end-of-file, driver addresses
        self.root = self.entry(pos)

    def u8(self, p):
        return self.d[p]

    def u16(self, p):
        return struct.unpack_from("<H", self.d, p)[0]

    def u32(self, p):
        return struct.unpack_from("<I", self.d, p)[0]

    def u64(self, p):
        return struct.unpack_from("<Q", self.d, p)[0]

    def entry(self, p):
        """Symbol-table entry: (name offset, object header address, cache type, scratch)."""
        return self.u64(p), self.u64(p + 8), self.u32(p + 16), self.d[p + 24:p + 40]

    # ---- object headers (version 1) ----
    def messages(self, addr):
        d = self.d
        if d[addr] != 1:
            raise ValueError("object header version %d not supported" % d[addr])
        nmsg = self.u16(addr + 2)
        size = self.u32(addr + 8)
        blocks = [(addr + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            p, size = blocks.pop(0)
            end = p + size
            while p + 8 <= end and len(out) < nmsg:
                mtype, msize = self.u16(p), self.u16(p + 2)
                body = p + 8
                if mtype == 0x10:       # continuation
                    blocks.append((self.u64(body), self.u64(body + 8)))
                out.append((mtype, body, msize))
                p = body + msize
        return out

    def heap_name(self, heap_addr, off):
        if self.d[heap_addr:heap_addr + 4] != b"HEAP":
            raise ValueError("bad local heap")
        seg = self.u64(heap_addr + 24)
        s = seg + off
        e = self.d.index(b"\0", s)
        return self.d[s:e].decode()

    def group_entries(self, btree, heap):
        """All (name, header address) pairs of an old-style group."""
        out = []
        stack = [btree]
        while stack:
            a = stack.pop()
            if self.d[a:a + 4] != b"TREE":
                raise ValueError("bad group B-tree node")
            level, used = self.d[a + 5], self.u16(a + 6)
            p = a + 24 + self.sl        # skip key 0
            for _ in range(used):
                child = self.u64(p)
                p += 8 + self.sl
                if level > 0:
                    stack.append(child)
                    continue
                if self.d[child:child + 4] != b"SNOD":
                    raise ValueError("bad symbol node")
                nsym = self.u16(child + 6)
                q = child + 8
                for _ in range(nsym):
                    noff, hdr, _, _ = self.entry(q)
                    out.append((self.heap_name(heap, noff), hdr))
                    q += 40
        return out

    # ---- datasets ----
    def dataset(self, msgs):
        shape, dtype, layout, filters = None, None, None, []
        for mtype, p, _ in msgs:
            if mtype == 0x01:           # dataspace
                ver, rank, flags = self.d[p], self.d[p + 1], self.d[p + 2]
                q = p + (8 if ver == 1 else 4)
                shape = tuple(self.u64(q + 8 * r) for r in range(rank))
            elif mtype == 0x03:         # datatype
                cls = self.d[p] & 0x0F
                bits = self.d[p + 1]
                size = self.u32(p + 4)
                big = bits & 1
                if cls == 1:
                    kind = "f"
                elif cls == 0:
                    kind = "i" if (bits & 0x08) else "u"
                else:
                    return None         # strings, compounds: not needed here
                dtype = np.dtype(("%s%s%d" % (">" if big else "<", kind, size)))
            elif mtype == 0x08:         # data layout
                ver = self.d[p]
                if ver != 3:
                    raise ValueError("layout version %d not supported" % ver)
                cls = self.d[p + 1]
                if cls == 1:
                    layout = ("contiguous", self.u64(p + 2), self.u64(p + 10))
                elif cls == 2:
                    rank = self.d[p + 2]
                    addr = self.u64(p + 3)
                    dims = [self.u32(p + 11 + 4 * r) for r in range(rank)]
                    layout = ("chunked", addr, dims)
                elif cls == 0:
                    size = self.u16(p + 2)
                    layout = ("compact", p + 4, size)
                else:
                    raise ValueError("layout class %d not supported" % cls)
            elif mtype == 0x0B:         # filter pipeline
                ver, nf = self.d[p], self.d[p + 1]
                q = p + (8 if ver == 1 else 2)
                for _ in range(nf):
                    fid = self.u16(q)
                    if ver == 1:
                        nlen, nval = self.u16(q + 2), self.u16(q + 6)
                        q += 8 + ((nlen + 7) // 8) * 8 + 4 * nval + (4 if nval % 2 else 0)
                    else:
                        nval = self.u16(q + 4)
                        q += 6 + 4 * nval
                    filters.append(fid)
        if shape is None or dtype is None or layout is None:
            return None
        count = int(np.prod(shape)) if shape else 1
        if layout[0] in ("contiguous", "compact"):
            raw = self.d[layout[1]:layout[1] + count * dtype.itemsize]
            return np.frombuffer(raw, dtype=dtype).reshape(shape).astype(dtype.newbyteorder("="))
        return self.chunked(layout[1], layout[2], shape, dtype, filters)

    def chunked(self, btree, cdims, shape, dtype, filters):
        rank = len(shape)
        out = np.zeros(shape, dtype=dtype.newbyteorder("="))
        cshape = tuple(cdims[:rank])
        stack = [btree]
        while stack:
            a = stack.pop()
            if self.d[a:a + 4] != b"TREE" or self.d[a + 4] != 1:
                raise ValueError("bad chunk B-tree node")
            level, used = self.d[a + 5], self.u16(a + 6)
            p = a + 24
            ksize = 8 + 8 * (rank + 1)
            for _ in range(used):
                csize, fmask = self.u32(p), self.u32(p + 4)
                offs = [self.u64(p + 8 + 8 * r) for r in range(rank)]
                child = self.u64(p + ksize)
                p += ksize + 8
                if level > 0:
                    stack.append(child)
                    continue
                raw = self.d[child:child + csize]
                for fid in reversed(filters):
                    if fid == 1:
                        raw = zlib.decompress(raw)
                    elif fid != 0:
                        raise ValueError("filter %d not supported" % fid)
                blk = np.frombuffer(raw[:int(np.prod(cshape)) * dtype.itemsize], dtype=dtype).reshape(cshape)
                sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cshape, shape))
                out[sl] = blk[tuple(slice(0, x.stop - x.start) for x in sl)]
        return out


def read(path):
    """Every dataset of an HDF5 file as {"group/name": array}."""
    with open(path, "rb") as fh:
        f = _File(fh.read())
    out = {}
    todo = [("", f.root[1])]
    while todo:
        prefix, hdr = todo.pop()
        msgs = f.messages(hdr)
        stab = [(p) for t, p, _ in msgs if t == 0x11]
        if stab:
            btree, heap = f.u64(stab[0]), f.u64(stab[0] + 8)
            for name, child in f.group_entries(btree, heap):
                todo.append((prefix + name + "/", child))
            continue
        arr = f.dataset(msgs)
        if arr is not None:
            out[prefix.rstrip("/")] = arr
    return out


if __name__ == "__main__":
    import sys
    for k, v in read(sys.argv[1]).items():
        print(k, v.shape, v.dtype, float(np.linalg.norm(v.astype(float))) if v.size else None)
