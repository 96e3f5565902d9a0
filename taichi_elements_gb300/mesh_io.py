"""Mesh and point-cloud files: taichi-dev/taichi_elements engine/mesh_io.py.

``load_mesh(fn, scale=1, offset=(0, 0, 0))`` returns the triangles of a PLY
mesh as an (n, 9) float32 array of vertex coordinates, scaled and offset
per axis (engine/mesh_io.py:5-22), ready for ``MPMSolver.add_mesh``.  The
reference parses with the ``plyfile`` package; this reader handles the
ASCII and binary (little- and big-endian) PLY forms directly: a ``vertex``
element with float ``x``, ``y``, ``z`` properties and a ``face`` element
whose vertex-index list holds triangles.  ``write_point_cloud`` writes the
binary point-cloud PLY of engine/mesh_io.py:25-44.
"""
from __future__ import annotations

import numpy as np

from .particle_io import write_point_cloud  # noqa: F401  (engine/mesh_io.py:25-44)

_PLY_TYPES = {
    'char': 'i1', 'int8': 'i1', 'uchar': 'u1', 'uint8': 'u1', 'short': 'i2', 'int16': 'i2', 'ushort': 'u2',
    'uint16': 'u2', 'int': 'i4', 'int32': 'i4', 'uint': 'u4', 'uint32': 'u4', 'float': 'f4', 'float32': 'f4',
    'double': 'f8', 'float64': 'f8'
}


def _parse_header(f):
    if f.readline().strip() != b'ply':
        raise ValueError('not a PLY file')
    fmt, elements = None, []
    while True:
        line = f.readline()
        if not line:
            raise ValueError('PLY header without end_header')
        words = line.decode('ascii', 'replace').split()
        if not words or words[0] in ('comment', 'obj_info'):
            continue
        if words[0] == 'format':
            fmt = words[1]
        elif words[0] == 'element':
            elements.append({'name': words[1], 'count': int(words[2]), 'props': []})
        elif words[0] == 'property':
            if words[1] == 'list':
                elements[-1]['props'].append((words[4], 'list', words[2], words[3]))
            else:
                elements[-1]['props'].append((words[2], words[1]))
        elif words[0] == 'end_header':
            return fmt, elements


def _read_binary(f, elements, order):
    data = {}
    for el in elements:
        props = el['props']
        if all(p[1] != 'list' for p in props):
            dt = np.dtype([(p[0], order + _PLY_TYPES[p[1]]) for p in props])
            data[el['name']] = np.frombuffer(f.read(dt.itemsize * el['count']), dt, el['count'])
            continue
        rows = []
        for _ in range(el['count']):
            row = {}
            for p in props:
                if p[1] == 'list':
                    ct = np.dtype(order + _PLY_TYPES[p[2]])
                    k = int(np.frombuffer(f.read(ct.itemsize), ct)[0])
                    it = np.dtype(order + _PLY_TYPES[p[3]])
                    row[p[0]] = np.frombuffer(f.read(it.itemsize * k), it, k)
                else:
                    t = np.dtype(order + _PLY_TYPES[p[1]])
                    row[p[0]] = np.frombuffer(f.read(t.itemsize), t)[0]
            rows.append(row)
        data[el['name']] = rows
    return data


def _read_ascii(f, elements):
    tokens = iter(f.read().split())
    data = {}
    for el in elements:
        props = el['props']
        if all(p[1] != 'list' for p in props):
            cols = {p[0]: np.empty(el['count'], _PLY_TYPES[p[1]]) for p in props}
            for i in range(el['count']):
                for p in props:
                    cols[p[0]][i] = float(next(tokens))
            data[el['name']] = cols
            continue
        rows = []
        for _ in range(el['count']):
            row = {}
            for p in props:
                if p[1] == 'list':
                    k = int(next(tokens))
                    row[p[0]] = np.array([int(next(tokens)) for _ in range(k)])
                else:
                    row[p[0]] = float(next(tokens))
            rows.append(row)
        data[el['name']] = rows
    return data


def load_mesh(fn, scale=1, offset=(0, 0, 0)):
    """engine/mesh_io.py:5-22: triangles (n, 9) float32 of a PLY mesh."""
    if isinstance(scale, (int, float)):
        scale = (scale, scale, scale)
    print(f'loading {fn}')
    with open(fn, 'rb') as f:
        fmt, elements = _parse_header(f)
        if fmt == 'ascii':
            data = _read_ascii(f, elements)
        elif fmt in ('binary_little_endian', 'binary_big_endian'):
            data = _read_binary(f, elements, '<' if fmt == 'binary_little_endian' else '>')
        else:
            raise ValueError(f'unknown PLY format {fmt}')
    vert = data['vertex']
    x, y, z = (np.asarray(vert[c], np.float64) for c in ('x', 'y', 'z'))
    faces = data['face']
    key = next(k for k in faces[0].keys() if 'vertex' in k) if faces else 'vertex_indices'
    triangles = np.zeros((len(faces), 9), dtype=np.float32)
    for i, face in enumerate(faces):
        idx = face[key]
        assert len(idx) == 3
        for d in range(3):
            triangles[i, d * 3 + 0] = x[idx[d]] * scale[0] + offset[0]
            triangles[i, d * 3 + 1] = y[idx[d]] * scale[1] + offset[1]
            triangles[i, d * 3 + 2] = z[idx[d]] * scale[2] + offset[2]
    return triangles
