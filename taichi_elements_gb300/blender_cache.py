"""The Blender add-on's particle cache: taichi-dev/taichi_elements
blender/particles_io.py (format version 1) and the frame writer of
blender/operators.py:228-247 (``save_particles``).

One cache frame is a header file ``particles_NNNNNN.bin`` — the format
version and the particle count as native ``uint32``, then for each of the five
attributes (position, velocity, colour, material, emitter id) the length and
the UTF-8 bytes of its file name — and five raw attribute files
``particles_NNNNNN_{pos,vel,col,mat,emt}.bin`` (float32 (n,3) positions and
velocities, int32 colours, materials and emitter ids, C order).

``save_particles(solver, cache_folder, frame)`` writes a frame of a GB300
solver: the five attributes are gathered into original particle order on the
device (one kernel per attribute, ``particle_info``) and copied to the host
once.  ``read_pars`` reads a frame back (the reference resolves file names
with ``bpy.path.abspath``; here they are joined to the folder).
"""
from __future__ import annotations

import os
import struct

import numpy as np

PARS_FMT_VER = 1

POS, VEL, COL, MAT, EMT = 0, 1, 2, 3, 4
attr_types = {POS: np.float32, VEL: np.float32, COL: np.int32, EMT: np.int32, MAT: np.int32}
attr_names = {POS: 'pos', VEL: 'vel', COL: 'col', MAT: 'mat', EMT: 'emt'}
attr_count = len(attr_names)


def write_pars(par_data, fpath, fname):
    """blender/particles_io.py:40-61: writes the five attribute files at
    ``{fpath}_{name}.bin`` and returns the header bytes (the caller writes
    them to ``{fpath}.bin``)."""
    data = bytearray()
    data.extend(struct.pack('I', PARS_FMT_VER))
    data.extend(struct.pack('I', par_data[POS].shape[0]))
    for attr_id in range(attr_count):
        name = bytes('{}_{}.bin'.format(fname, attr_names[attr_id]), 'utf-8')
        data.extend(struct.pack('I', len(name)))
        data.extend(struct.pack('{}s'.format(len(name)), name))
    for attr_id in range(attr_count):
        np.asarray(par_data[attr_id]).tofile('{}_{}.bin'.format(fpath, attr_names[attr_id]))
    return data


def read_pars(file_path, caches=None, folder=None):
    """blender/particles_io.py:64-98: the attributes of one cache frame as
    flat arrays keyed by attribute id (stored in ``caches[folder]`` when a
    dict is given, as the reference does)."""
    folder = os.path.dirname(file_path) if folder is None else folder
    with open(file_path, 'rb') as f:
        data = f.read()
    offs = 0
    ver = struct.unpack('I', data[offs:offs + 4])[0]
    offs += 4
    if ver != PARS_FMT_VER:
        raise ValueError('Unsupported particles format version: {0}'.format(ver))
    offs += 4  # particle count (the attribute files carry their own length)
    out = {}
    for attr_id in range(attr_count):
        n = struct.unpack('I', data[offs:offs + 4])[0]
        offs += 4
        name = str(struct.unpack('{}s'.format(n), data[offs:offs + n])[0], 'utf-8')
        offs += n
        out[attr_id] = np.fromfile(os.path.join(folder, name), dtype=attr_types[attr_id])
    if caches is not None:
        caches[folder] = out
    return out


def save_particles(solver, cache_folder, frame):
    """blender/operators.py:228-247 for a GB300 solver: one cache frame of
    all particles in original order.  Emitter ids are zero unless the solver
    was made with ``use_emitter_id=True``.  Returns the header path."""
    os.makedirs(cache_folder, exist_ok=True)
    fname = 'particles_{0:0>6}'.format(frame)
    fpath = os.path.join(cache_folder, fname)
    info = solver.particle_info()
    n = info['position'].shape[0]
    emt = info.get('emitter_ids', np.zeros(n, np.int32))
    par_data = {
        POS: np.ascontiguousarray(info['position'], np.float32),
        VEL: np.ascontiguousarray(info['velocity'], np.float32),
        COL: np.ascontiguousarray(info['color'], np.int32),
        MAT: np.ascontiguousarray(info['material'], np.int32),
        EMT: np.ascontiguousarray(emt, np.int32),
    }
    data = write_pars(par_data, fpath, fname)
    with open(fpath + '.bin', 'wb') as f:
        f.write(data)
    return fpath + '.bin'
