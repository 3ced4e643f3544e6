"""Keras HDF5 weight files (model.save_weights / load_weights) without h5py.

A reader for the subset of HDF5 that Keras' ``save_weights`` produces through
h5py's default file format: superblock version 0, version-1 object headers
(with continuation blocks), groups stored as symbol tables (version-1 B-trees
of symbol-table nodes and a local heap for the names), attributes holding
fixed-length string arrays (``layer_names``, ``weight_names``) and datasets
of little-endian IEEE floats with contiguous or compact layout. Anything
outside that subset raises ``ValueError``.

``read_keras_weights(path)`` returns the weighted layers in the order of the
file's ``layer_names`` attribute, each as ``(layer name, [(weight name,
array), ...])`` in the order of the layer's ``weight_names`` attribute.
``load_conv_net_autoregressive_2d(machine, path)`` maps such a file onto a
``ConvNetAutoregressive2D``: taken in creation order (the index Keras appends
to a layer class's name), per causal conv the vertical 3x3, the
horizontal 1x3, the two 1x1 convs (x, y) and the combining 3x3
(machines/conv_net_autoregressive_2D.py:33-51), each WeightNormalization
layer holding kernel, bias and g (deepar/layers/wrappers.py:83-105), then the
plain 1x1 output conv (:73). This is how the reference's published models
(experiments/weights/*.h5) are evaluated here.
"""
import numpy as np
import torch


class _H5:
    def __init__(self, data):
        self.b = data
        if data[:8] != b"\x89HDF\r\n\x1a\n":
            raise ValueError("not an HDF5 file")
        if data[8] != 0:
            raise ValueError("HDF5 superblock version %d is not supported (0 only)" % data[8])
        self.so, self.sl = data[13], data[14]
        if self.so != 8 or self.sl != 8:
            raise ValueError("HDF5 offsets/lengths of 8 bytes only")
        self.base = self.u(24, 8)
        root = 56  # root group symbol-table entry
        self.root = self.u(root + 8, 8)

    def u(self, off, n):
        return int.from_bytes(self.b[off:off + n], "little")

    def addr(self, a):
        return self.base + a

    # ---- object headers
    def messages(self, oh):
        """(type, data offset, size) of the messages of an object header (version 1)."""
        a = self.addr(oh)
        if self.b[a] != 1:
            raise ValueError("object header version %d is not supported (1 only)" % self.b[a])
        n = self.u(a + 2, 2)
        size = self.u(a + 8, 4)
        blocks = [(a + 16, size)]
        out = []
        while blocks and len(out) < n:
            start, length = blocks.pop(0)
            p, end = start, start + length
            while p + 8 <= end and len(out) < n:
                mtype, msize = self.u(p, 2), self.u(p + 2, 2)
                d = p + 8
                if mtype == 0x10:  # continuation
                    blocks.append((self.addr(self.u(d, 8)), self.u(d + 8, 8)))
                out.append((mtype, d, msize))
                p = d + msize
        return out

    def dataspace(self, d):
        ver, rank, flags = self.b[d], self.b[d + 1], self.b[d + 2]
        p = d + 8 if ver == 1 else d + 4
        if ver not in (1, 2):
            raise ValueError("dataspace version %d" % ver)
        if ver == 2 and self.b[d + 3] == 0:  # scalar
            return ()
        return tuple(self.u(p + 8 * i, 8) for i in range(rank))

    def datatype(self, d):
        cls = self.b[d] & 0x0F
        bits = self.b[d + 1]
        size = self.u(d + 4, 4)
        if cls == 1:  # floating point
            if bits & 1:
                raise ValueError("big-endian floats are not supported")
            # (other sizes, e.g. the 16-byte floats of an empty weight_names, as opaque bytes)
            return {4: np.dtype("<f4"), 8: np.dtype("<f8"), 2: np.dtype("<f2")}.get(size, np.dtype("V%d" % size))
        if cls == 0:  # fixed-point integer
            signed = bool(bits & 0x08)
            return np.dtype(("<i%d" if signed else "<u%d") % size)
        if cls == 3:  # fixed-length string
            return np.dtype("S%d" % size)
        if cls == 9 and (bits & 0x0F) == 1:  # variable-length string (global heap)
            return "vlen-str"
        raise ValueError("HDF5 datatype class %d is not supported" % cls)

    def vlen_strings(self, p, count):
        """Elements (length, global heap collection, object index) -> str."""
        out = []
        for i in range(count):
            e = p + 16 * i
            n, coll, idx = self.u(e, 4), self.u(e + 4, 8), self.u(e + 12, 4)
            c = self.addr(coll)
            if self.b[c:c + 4] != b"GCOL":
                raise ValueError("bad global heap collection")
            end = c + self.u(c + 8, 8)
            q = c + 16
            val = None
            while q + 16 <= end:
                oid, osz = self.u(q, 2), self.u(q + 8, 8)
                if oid == 0:
                    break
                if oid == idx:
                    val = self.b[q + 16:q + 16 + n].decode()
                    break
                q += 16 + (osz + 7) // 8 * 8
            if val is None:
                raise ValueError("global heap object %d not found" % idx)
            out.append(val)
        return out

    def attributes(self, oh):
        out = {}
        for mtype, d, _ in self.messages(oh):
            if mtype != 0x0C:
                continue
            ver = self.b[d]
            nsz, tsz, ssz = self.u(d + 2, 2), self.u(d + 4, 2), self.u(d + 6, 2)
            if ver == 1:
                pad = lambda x: (x + 7) // 8 * 8
                p = d + 8
                name = self.b[p:p + nsz].split(b"\0")[0].decode()
                p += pad(nsz)
                dt = self.datatype(p)
                p += pad(tsz)
                shape = self.dataspace(p)
                p += pad(ssz)
            elif ver in (2, 3):
                p = d + 8 + (1 if ver == 3 else 0)
                name = self.b[p:p + nsz].split(b"\0")[0].decode()
                p += nsz
                dt = self.datatype(p)
                p += tsz
                shape = self.dataspace(p)
                p += ssz
            else:
                raise ValueError("attribute message version %d" % ver)
            count = int(np.prod(shape)) if shape else 1
            if isinstance(dt, str):
                vals = self.vlen_strings(p, count)
                out[name] = np.array(vals, dtype=object).reshape(shape) if shape else vals[0]
                continue
            arr = np.frombuffer(self.b, dtype=dt, count=count, offset=p)
            out[name] = arr.reshape(shape) if shape else arr[0]
        return out

    # ---- groups
    def children(self, oh):
        """name -> object header address of a symbol-table group."""
        for mtype, d, _ in self.messages(oh):
            if mtype == 0x11:
                btree, heap = self.u(d, 8), self.u(d + 8, 8)
                break
        else:
            raise ValueError("group without a symbol table (new-style groups are not supported)")
        h = self.addr(heap)
        if self.b[h:h + 4] != b"HEAP":
            raise ValueError("bad local heap")
        heap_data = self.addr(self.u(h + 24, 8))
        out = {}

        def walk(node):
            a = self.addr(node)
            if self.b[a:a + 4] != b"TREE":
                raise ValueError("bad B-tree node")
            level, used = self.b[a + 5], self.u(a + 6, 2)
            p = a + 24 + 8  # past the header and key 0
            for _ in range(used):
                child = self.u(p, 8)
                p += 16  # child address, next key
                if level > 0:
                    walk(child)
                else:
                    s = self.addr(child)
                    if self.b[s:s + 4] != b"SNOD":
                        raise ValueError("bad symbol-table node")
                    for k in range(self.u(s + 6, 2)):
                        e = s + 8 + 40 * k
                        name_off, obj = self.u(e, 8), self.u(e + 8, 8)
                        q = heap_data + name_off
                        name = self.b[q:self.b.index(b"\0", q)].decode()
                        out[name] = obj

        walk(btree)
        return out

    def dataset(self, oh):
        dt = shape = None
        for mtype, d, _ in self.messages(oh):
            if mtype == 0x01:
                shape = self.dataspace(d)
            elif mtype == 0x03:
                dt = self.datatype(d)
            elif mtype == 0x08:
                ver = self.b[d]
                if ver != 3:
                    raise ValueError("data layout version %d (3 only)" % ver)
                cls = self.b[d + 1]
                if cls == 1:
                    data_at, nbytes = self.u(d + 2, 8), self.u(d + 10, 8)
                    off = self.addr(data_at) if data_at != 0xFFFFFFFFFFFFFFFF else None
                elif cls == 0:
                    nbytes = self.u(d + 2, 2)
                    off = d + 4
                else:
                    raise ValueError("chunked datasets are not supported")
        if dt is None or shape is None:
            raise ValueError("dataset without datatype or dataspace")
        count = int(np.prod(shape)) if shape else 1
        if off is None:
            return np.zeros(shape, dtype=dt)
        return np.frombuffer(self.b, dtype=dt, count=count, offset=off).reshape(shape).copy()

    def lookup(self, path):
        oh = self.root
        for part in [x for x in path.split("/") if x]:
            oh = self.children(oh)[part]
        return oh


def _strings(a):
    return [x.decode() if isinstance(x, bytes) else str(x) for x in np.asarray(a).reshape(-1)]


def read_keras_weights(path):
    with open(path, "rb") as f:
        h = _H5(f.read())
    attrs = h.attributes(h.root)
    grp = h.root
    if "layer_names" not in attrs and "model_weights" in h.children(h.root):  # model.save() files
        grp = h.children(h.root)["model_weights"]
        attrs = h.attributes(grp)
    if "layer_names" not in attrs:
        raise ValueError("no layer_names attribute: not a Keras weight file")
    layers = []
    top = h.children(grp)
    for lname in _strings(attrs["layer_names"]):
        g = top[lname]
        wnames = _strings(h.attributes(g).get("weight_names", []))
        if not wnames:
            continue
        weights = []
        for wn in wnames:
            oh = g
            for part in wn.split("/"):
                oh = h.children(oh)[part]
            weights.append((wn, h.dataset(oh)))
        layers.append((lname, weights))
    return layers


def _by_role(weights):
    out = {}
    for name, arr in weights:
        base = name.split("/")[-1].split(":")[0]
        out[base] = arr
    return out


def _creation_order(layers):
    """Keras names a layer class's instances <name>, <name>_1, <name>_2, ... in
    creation order, while a file lists layers in graph order (which differs for
    the final causal conv). Weight-normalised convs sorted by that index, then
    the plain output conv."""
    def key(item):
        name = item[0]
        base, _, idx = name.rpartition("_")
        if not idx.isdigit():
            base, idx = name, "0"
        return (0 if base == "weight_normalization" else 1, int(idx))
    return sorted(layers, key=key)


def keras_weights_to_flat(layers, layout):
    """Flat FP32 parameter vector of a ConvNetAutoregressive2D ``layout``
    (machines.ar2d_param_layout) from the weighted layers of a Keras file."""
    layers = _creation_order(layers)
    convs = [name[: -len(".kernel")] for name, _, _ in layout if name.endswith(".kernel")]
    if len(layers) != len(convs):
        raise ValueError("the file holds %d weighted layers, the machine %d convolutions" % (len(layers), len(convs)))
    index = {name: (tuple(shape), off) for name, shape, off in layout}
    total = max(off + int(np.prod(shape)) for _, shape, off in layout)
    flat = np.zeros(total, dtype=np.float32)
    for (lname, weights), conv in zip(layers, convs):
        roles = _by_role(weights)
        for role in ("kernel", "bias", "g"):
            key = conv + "." + role
            if key not in index:
                if role in roles:
                    raise ValueError("layer %s holds %s, which %s does not have" % (lname, role, conv))
                continue
            if role not in roles:
                raise ValueError("layer %s has no %s for %s" % (lname, role, conv))
            shape, off = index[key]
            arr = np.asarray(roles[role], dtype=np.float32)
            if tuple(arr.shape) != shape:
                raise ValueError("%s: file shape %s, machine shape %s" % (key, arr.shape, shape))
            flat[off:off + arr.size] = arr.reshape(-1)
    return flat


def load_conv_net_autoregressive_2d(machine, path):
    """Loads a Keras weight file of the reference's ConvNetAutoregressive2D
    into ``machine`` (same depth, channels and weight normalisation)."""
    flat = keras_weights_to_flat(read_keras_weights(path), machine.layout)
    if flat.size != machine.params.numel():
        raise ValueError("layout size %d, machine parameters %d" % (flat.size, machine.params.numel()))
    machine.params.copy_(torch.from_numpy(flat).to(machine.params.device))
    machine.params_updated()
    return machine
