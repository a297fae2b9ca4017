"""HDF5 + XDMF output of simulation fields (pylbm/hdf5.py ``H5File``).

pylbm writes its results with h5py and an XDMF sidecar for ParaView/VisIt.
h5py is not available to this backend, so the file is written here directly,
single process (the MPI gather of the reference has nothing to gather), in the
layout h5py gives the reference's own files (the ones in pylbm's
tests/reference/): superblock version 0, a root group with a version-1
B-tree and a local heap, and one contiguous little-endian float64 dataset per
field whose object header holds the dataspace, datatype, fill-value, layout
and modification-time messages.  The coordinates go in ``x_0``, ``x_1``,
``x_2`` and the fields are stored transposed (``global_size[::-1]``), as
pylbm does (pylbm/hdf5.py:167, :204-206).

The fields come from ``Simulation.m`` / ``Simulation.fields``, which read all
conserved moments with one device-to-host copy.
"""
import os
import struct
import time

import numpy as np

_UNDEF = 0xFFFFFFFFFFFFFFFF
_LEAF_K = 16         # group leaf node K (up to 2K datasets in the one symbol table node)
_INTERNAL_K = 16


def _pad8(b):
    return b + b"\0" * (-len(b) % 8)


def _message(mtype, body, flags=0):
    body = _pad8(body)
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _object_header(messages):
    data = b"".join(messages)
    return struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(data)) + data


def _dataspace(shape):
    body = struct.pack("<BBB5x", 1, len(shape), 1)
    body += b"".join(struct.pack("<Q", n) for n in shape)
    body += b"".join(struct.pack("<Q", n) for n in shape)  # maximum sizes
    return _message(0x0001, body)


def _float64_type():
    # class 1 (floating point), version 1; little endian, IEEE normalisation,
    # sign at bit 63; offset 0, precision 64, exponent 52/11, mantissa 0/52, bias 1023
    body = struct.pack("<B3BI", 0x11, 0x20, 0x3F, 0x00, 8)
    body += struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
    return _message(0x0003, body, flags=1)


def _fill_value():
    # version 2: late allocation, fill written never... (as h5py writes it), no value
    return _message(0x0005, struct.pack("<BBBBI", 2, 2, 2, 1, 0), flags=1)


def _layout(addr, size):
    return _message(0x0008, struct.pack("<BBQQ", 3, 1, addr, size))


def _mtime():
    return _message(0x0012, struct.pack("<B3xI", 1, int(time.time()) & 0xFFFFFFFF))


def write_h5(path, datasets):
    """Write {name: float64 array} as datasets of the root group of a new HDF5 file."""
    names = sorted(datasets)  # symbol table entries are kept in name order
    if len(names) > 2 * _LEAF_K:
        raise ValueError(f"at most {2 * _LEAF_K} datasets per file")
    arrays = [np.ascontiguousarray(datasets[n], dtype="<f8") for n in names]

    # local heap: "" at 0, then the names, 8-byte aligned
    heap_data = b"\0" * 8
    offsets = []
    for n in names:
        offsets.append(len(heap_data))
        heap_data += _pad8(n.encode() + b"\0")

    sb_size = 24 + 4 * 8 + 40
    root_hdr_addr = sb_size
    root_hdr_len = len(_object_header([_message(0x0011, b"\0" * 16)]))
    btree_addr = root_hdr_addr + root_hdr_len
    btree_len = 8 + 2 * 8 + (2 * _LEAF_K + 1) * 8 + 2 * _LEAF_K * 8
    heap_addr = btree_addr + btree_len
    heap_hdr_len = 32
    heap_seg_addr = heap_addr + heap_hdr_len
    snod_addr = heap_seg_addr + len(heap_data)
    snod_len = 8 + 2 * _LEAF_K * 40
    cursor = snod_addr + snod_len
    headers, data_addrs = [], []
    for a in arrays:
        # the rank enters the dataspace message: each header has its own size
        hdr_len = len(_object_header([_dataspace(a.shape), _float64_type(), _fill_value(), _layout(0, 0),
                                      _mtime()]))
        headers.append(cursor)
        cursor += hdr_len
    for a in arrays:
        cursor += -cursor % 8
        data_addrs.append(cursor)
        cursor += a.nbytes
    eof = cursor

    out = bytearray(eof)
    # superblock (version 0)
    sb = b"\x89HDF\r\n\x1a\n" + struct.pack("<BBBBBBBBHHI", 0, 0, 0, 0, 0, 8, 8, 0, _LEAF_K, _INTERNAL_K, 0)
    sb += struct.pack("<QQQQ", 0, _UNDEF, eof, _UNDEF)
    sb += struct.pack("<QQI4xQQ", 0, root_hdr_addr, 1, btree_addr, heap_addr)
    out[0:len(sb)] = sb
    root = _object_header([_message(0x0011, struct.pack("<QQ", btree_addr, heap_addr))])
    out[root_hdr_addr:root_hdr_addr + len(root)] = root
    # group B-tree: one leaf child (the symbol table node); key = heap offset of its last name
    bt = b"TREE" + struct.pack("<BBH", 0, 0, 1) + struct.pack("<QQ", _UNDEF, _UNDEF)
    bt += struct.pack("<QQQ", 0, snod_addr, offsets[-1] if offsets else 0)
    out[btree_addr:btree_addr + len(bt)] = bt
    heap = b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap_data), _UNDEF, heap_seg_addr)
    out[heap_addr:heap_addr + len(heap)] = heap
    out[heap_seg_addr:heap_seg_addr + len(heap_data)] = heap_data
    sn = b"SNOD" + struct.pack("<BBH", 1, 0, len(names))
    for off, hdr in zip(offsets, headers):
        sn += struct.pack("<QQI4x16x", off, hdr, 0)
    out[snod_addr:snod_addr + len(sn)] = sn
    for a, hdr, addr in zip(arrays, headers, data_addrs):
        h = _object_header([_dataspace(a.shape), _float64_type(), _fill_value(), _layout(addr, a.nbytes), _mtime()])
        out[hdr:hdr + len(h)] = h
        out[addr:addr + a.nbytes] = a.tobytes()
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "wb") as fh:
        fh.write(bytes(out))
    os.replace(tmp, path)


class H5File:
    """pylbm.H5File for one process (pylbm/hdf5.py:20-322).

    ``H5File(mpi_topo, filename, path, timestep)``; ``set_grid(x, y, z)``,
    ``add_scalar(name, array_or_function, *args)``,
    ``add_vector(name, [arrays] or function, *args)``, ``save()`` writes
    ``<path>/<name>[_<timestep>].h5`` and the ``.xdmf`` description.
    ``mpi_topo`` is accepted for signature compatibility and not used.
    """

    def __init__(self, mpi_topo=None, filename="output", path="", timestep=None, init_xdmf=False):
        prefix = f"_{timestep}" if timestep is not None else ""
        name, _ = os.path.splitext(filename)
        self.path = path or "."
        self.filename = name + prefix
        self.h5filename = self.filename + ".h5"
        os.makedirs(self.path, exist_ok=True)
        self.global_size = None
        self.dim = None
        self.origin = self.dx = None
        self._datasets = {}
        self.scalars = {}
        self.vectors = {}

    def set_grid(self, x, y=None, z=None):
        coords = [np.asarray(c, dtype=np.float64) for c in (x, y, z) if c is not None]
        self.dim = len(coords)
        self.origin = [c[0] for c in coords]
        self.dx = [c[1] - c[0] if c.size > 1 else 0.0 for c in coords]
        self.global_size = [c.size for c in coords]
        for i, c in enumerate(coords):
            self._datasets[f"x_{i}"] = c

    def _field(self, f, fargs):
        data = np.asarray(f if isinstance(f, np.ndarray) else f(*fargs), dtype=np.float64)
        if list(data.shape) != self.global_size:
            raise ValueError(f"field of shape {data.shape} on a grid of size {self.global_size}")
        return data.T

    def add_scalar(self, name, f, *fargs):
        self._datasets[name] = self._field(f, fargs)
        self.scalars[name] = f"{self.h5filename}:/{name}"

    def add_vector(self, name, f, *fargs):
        datas = f if isinstance(f, list) else f(*fargs)
        comps = [self._field(d, ()) for d in datas]
        while len(comps) < 3:  # pylbm stores vectors with 3 components
            comps.append(np.zeros_like(comps[0]))
        self._datasets[name] = np.stack(comps, axis=-1)
        self.vectors[name] = f"{self.h5filename}:/{name}"

    def save(self):
        write_h5(os.path.join(self.path, self.h5filename), self._datasets)
        dims = " ".join(map(str, self.global_size))
        rdims = " ".join(map(str, self.global_size[::-1]))
        mesh, geo = ("2DRectMesh", "VXVY") if self.dim == 2 else ("3DRectMesh", "VXVYVZ")
        lines = ['<?xml version="1.0" ?>', '<!DOCTYPE Xdmf SYSTEM "Xdmf.dtd" []>', "<Xdmf>", " <Domain>",
                 '  <Grid Name="Structured Grid" GridType="Uniform">',
                 f'   <Topology TopologyType="{mesh}" NumberOfElements="{dims}"/>',
                 f'   <Geometry GeometryType="{geo}">']
        for i in range(self.dim):
            lines += [f'    <DataItem Format="HDF" Dimensions="{self.global_size[i]}">',
                      f"     {self.h5filename}:/x_{i}", "    </DataItem>"]
        lines.append("   </Geometry>")
        for k, v in self.scalars.items():
            lines += [f'   <Attribute Name="{k}" AttributeType="Scalar" Center="Node">',
                      f'    <DataItem Format="HDF" Dimensions="{rdims}">', f"     {v}", "    </DataItem>",
                      "   </Attribute>"]
        for k, v in self.vectors.items():
            lines += [f'   <Attribute Name="{k}" AttributeType="Vector" Center="Node">',
                      f'    <DataItem Format="HDF" Dimensions="{rdims} 3">', f"     {v}", "    </DataItem>",
                      "   </Attribute>"]
        lines += ["  </Grid>", " </Domain>", "</Xdmf>"]
        with open(os.path.join(self.path, self.filename + ".xdmf"), "w") as fh:
            fh.write("\n".join(lines) + "\n")
