"""An independent HDF5 encoder for reader tests (test helper). It writes the
structures the C++ writer does not produce — superblock v2, version-2 object
headers with compact link messages, chunked storage indexed by a v1 B-tree with
shuffle + deflate filters, big-endian / float64 / integer element types, and a
version-1 object header split by a continuation message — following the HDF5
File Format Specification. Checksums of v2 structures are written as zero (the
reader under test does not verify them)."""
import struct
import zlib

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


class Buf:
    def __init__(self):
        self.b = bytearray()

    def put(self, data):
        self.b += data

    def u(self, v, n):
        self.b += int(v).to_bytes(n, "little")

    def pad(self, a=8):
        while len(self.b) % a:
            self.b.append(0)

    def here(self):
        return len(self.b)

    def patch(self, pos, v, n=8):
        self.b[pos:pos + n] = int(v).to_bytes(n, "little")


def dtype_bytes(dt, array3=False):
    dt = np.dtype(dt)
    big = dt.byteorder == ">" or (dt.byteorder == "=" and False)
    if dt.kind == "f":
        size = dt.itemsize
        mant, expo, bias = (23, 8, 127) if size == 4 else (52, 11, 1023)
        body = struct.pack("<BBBBI", 0x11, (1 if big else 0) | 0x20, size * 8 - 1, 0, size)
        body += struct.pack("<HHBBBBI", 0, size * 8, mant, expo, 0, mant, bias)
    else:
        size = dt.itemsize
        body = struct.pack("<BBBBI", 0x10, (1 if big else 0) | (0x08 if dt.kind == "i" else 0), 0, 0, size)
        body += struct.pack("<HH", 0, size * 8)
    if array3:
        return struct.pack("<BBBBI", 0x3A, 0, 0, 0, 3 * size) + struct.pack("<BI", 1, 3) + body  # array v3
    return body


def _msg_v2(t, body):
    return struct.pack("<BHB", t, len(body), 0) + body


def _ohdr_v2(msgs):
    body = b"".join(msgs)
    return b"OHDR" + bytes([2, 0x02]) + struct.pack("<I", len(body)) + body + b"\0\0\0\0"


def write_v2_chunked(path, data, chunk, filters=("shuffle", "deflate"), array3=False, fanout=None):
    """Superblock v2, v2 object headers, chunked + filtered dataset /data.
    fanout: at most this many entries per v1 B-tree node, so that many chunks
    give a tree of several levels (libhdf5 writes 2K = 64 per node by default);
    None: one leaf node holding every chunk."""
    data = np.ascontiguousarray(data)
    shape = data.shape[:-1] if array3 else data.shape
    rank = len(shape)
    es = data.dtype.itemsize * (3 if array3 else 1)
    f = Buf()
    f.put(b"\x89HDF\r\n\x1a\n" + bytes([2, 8, 8, 0]))
    f.u(0, 8)
    f.u(UNDEF, 8)
    eof_pos = f.here()
    f.u(0, 8)
    root_pos = f.here()
    f.u(0, 8)
    f.u(0, 4)
    # chunks
    nch = [(shape[k] + chunk[k] - 1) // chunk[k] for k in range(rank)]
    entries = []
    for idx in np.ndindex(*nch):
        origin = [idx[k] * chunk[k] for k in range(rank)]
        full = np.zeros(tuple(chunk) + ((3,) if array3 else ()), data.dtype)
        sl = tuple(slice(origin[k], min(origin[k] + chunk[k], shape[k])) for k in range(rank))
        part = data[sl]
        full[tuple(slice(0, s) for s in part.shape[:rank])] = part
        raw = full.tobytes()
        if "shuffle" in filters:
            a = np.frombuffer(raw, np.uint8).reshape(-1, data.dtype.itemsize)
            raw = a.T.tobytes()
        if "deflate" in filters:
            raw = zlib.compress(raw, 4)
        f.pad()
        addr = f.here()
        f.put(raw)
        entries.append((origin, len(raw), addr))
    # chunk B-tree: leaves of chunk entries, then parent levels of node entries
    # (each entry: key = chunk size, filter mask and offsets of the first chunk
    # below it; child address), each node closed by the key of its upper bound
    def node(level, items, upper):
        f.pad()
        at = f.here()
        f.put(b"TREE" + bytes([1, level]) + struct.pack("<H", len(items)))
        f.u(UNDEF, 8)
        f.u(UNDEF, 8)
        for origin, size, addr in items:
            f.put(struct.pack("<II", size, 0) + b"".join(struct.pack("<Q", o) for o in origin + [0]))
            f.u(addr, 8)
        f.put(struct.pack("<II", 0, 0) + b"".join(struct.pack("<Q", s) for s in upper + [0]))
        return at

    level, items = 0, entries
    m = fanout or max(len(entries), 1)
    while True:
        groups = [items[i:i + m] for i in range(0, len(items), m)]
        addrs = [node(level, g, list(shape)) for g in groups]
        if len(groups) == 1:
            btree = addrs[0]
            break
        items = [(g[0][0], g[0][1], a) for g, a in zip(groups, addrs)]
        level += 1
    # dataset header
    space = struct.pack("<BBBB", 2, rank, 0, 1) + b"".join(struct.pack("<Q", s) for s in shape)
    layout = struct.pack("<BBB", 3, 2, rank + 1) + struct.pack("<Q", btree) + \
        b"".join(struct.pack("<I", c) for c in chunk) + struct.pack("<I", es)
    fl = []
    if "shuffle" in filters:
        fl.append(struct.pack("<HHH", 2, 0, 1) + struct.pack("<I", data.dtype.itemsize))
    if "deflate" in filters:
        fl.append(struct.pack("<HHH", 1, 0, 1) + struct.pack("<I", 4))
    msgs = [_msg_v2(1, space), _msg_v2(3, dtype_bytes(data.dtype, array3)), _msg_v2(8, layout)]
    if fl:
        msgs.append(_msg_v2(0x0B, struct.pack("<BB", 2, len(fl)) + b"".join(fl)))
    f.pad()
    ds = f.here()
    f.put(_ohdr_v2(msgs))
    # root group: link info (no dense storage) + a link message to /data
    f.pad()
    root = f.here()
    linfo = struct.pack("<BB", 0, 0) + struct.pack("<QQ", UNDEF, UNDEF)
    link = struct.pack("<BBB", 1, 0, 4) + b"data" + struct.pack("<Q", ds)
    other = struct.pack("<BBB", 1, 0, 5) + b"other" + struct.pack("<Q", ds)
    f.put(_ohdr_v2([_msg_v2(2, linfo), _msg_v2(6, other), _msg_v2(6, link)]))
    f.patch(root_pos, root)
    f.patch(eof_pos, f.here())
    open(path, "wb").write(bytes(f.b))


def write_v0_continuation(path, data):
    """Superblock v0 whose root entry carries no cached symbol table (the
    reader must read the root object header), and a v1 dataset header whose
    layout message sits in a continuation block; contiguous big-endian data."""
    data = np.ascontiguousarray(data)
    f = Buf()
    f.put(b"\x89HDF\r\n\x1a\n" + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0))
    f.u(0, 8)
    f.u(UNDEF, 8)
    eof_pos = f.here()
    f.u(0, 8)
    f.u(UNDEF, 8)
    f.u(0, 8)
    root_pos = f.here()
    f.u(0, 8)
    f.u(0, 4)   # cache type 0: nothing cached
    f.u(0, 4)
    f.u(0, 16)
    # raw data
    f.pad()
    raw = f.here()
    f.put(data.tobytes())
    # local heap + SNOD + group B-tree
    f.pad()
    heap_data = f.here()
    hd = b"\0" * 8 + b"data\0\0\0\0"
    f.put(hd)
    f.pad()
    heap = f.here()
    f.put(b"HEAP\0\0\0\0" + struct.pack("<QQQ", len(hd), 1, heap_data))
    f.pad()
    snod = f.here()
    snod_entry_pos = f.here() + 8 + 8
    f.put(b"SNOD\x01\x00" + struct.pack("<H", 1) + struct.pack("<QQII", 8, 0, 0, 0) + b"\0" * 16)
    f.pad()
    btree = f.here()
    f.put(b"TREE\x00\x00" + struct.pack("<H", 1) + struct.pack("<QQ", UNDEF, UNDEF) +
          struct.pack("<QQQ", 0, snod, 8))
    # dataset v1 header: dataspace + datatype here, layout in a continuation block
    def msg_v1(t, body):
        body = body + b"\0" * ((8 - len(body) % 8) % 8)
        return struct.pack("<HHBxxx", t, len(body), 0) + body
    space = struct.pack("<BBBBI", 1, data.ndim, 0, 0, 0) + b"".join(struct.pack("<Q", s) for s in data.shape)
    layout = struct.pack("<BB", 3, 1) + struct.pack("<QQ", raw, data.nbytes)
    f.pad()
    cont = f.here()
    cont_block = msg_v1(8, layout)
    f.put(cont_block)
    f.pad()
    ds = f.here()
    first = msg_v1(1, space) + msg_v1(3, dtype_bytes(data.dtype)) + msg_v1(0x10, struct.pack("<QQ", cont, len(cont_block)))
    f.put(struct.pack("<BBHII", 1, 0, 3, 1, len(first)) + b"\0\0\0\0" + first)
    f.patch(snod_entry_pos, ds)
    # root group header with a symbol table message
    f.pad()
    root = f.here()
    f.put(struct.pack("<BBHII", 1, 0, 1, 1, 24) + b"\0\0\0\0" + msg_v1(0x11, struct.pack("<QQ", btree, heap)))
    f.patch(root_pos, root)
    f.patch(eof_pos, f.here())
    open(path, "wb").write(bytes(f.b))
