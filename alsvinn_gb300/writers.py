"""Output writers: the reference's NetCDF layout in the classic NetCDF
format, and a numpy (.npz) writer.

NetCDF (alsfvm/src/io/NetCDFWriter.cpp:35-200). One file named exactly the
basename, dimensions member (samples), time (saves), x, y and z for 3D grids;
coordinate variables member (int: 0 .. samples - 1), time (the writer's save
fractions (k + 1) / numberOfSaves, a leading 0 with writeInitialTimestep),
x, y[, z] (cell midpoints); and per conserved variable rho, E, mx, my[, mz]
(that order) a double array over (member, time, x, y[, z]). Each snapshot
writes a variable's interior cells in x-fastest order into the
(member, time) slab, as the reference does: a NetCDF reader therefore sees
the buffer laid out with the last dimension fastest. Burgers states, which
the reference's writer does not handle, are written as one variable u.

The reference writes NetCDF-4 (HDF5) through the NetCDF library, which is not
in this image; this writer produces the classic 64-bit-offset format (CDF-2),
which the same NetCDF library, netCDF4-python, xarray and scipy.io read with
the same names, shapes and values. Fill values are not written (the
reference sets NC_NOFILL); unwritten slabs read as zeros.
"""
import os
import struct

import numpy as np

from .initdata import cell_midpoints

NC_DIMENSION = 10
NC_VARIABLE = 11
NC_INT = 4
NC_DOUBLE = 6

STATE_NAMES = {
    "euler1": (("rho", 0), ("E", 2), ("mx", 1), ("my", None)),
    "euler2": (("rho", 0), ("E", 3), ("mx", 1), ("my", 2)),
    "euler3": (("rho", 0), ("E", 4), ("mx", 1), ("my", 2), ("mz", 3)),
    "burgers": (("u", 0),),
}


def _name(s):
    b = s.encode()
    return struct.pack(">i", len(b)) + b + b"\0" * (-len(b) % 4)


class NetCDFWriter:
    """Creates the file on construction (header, coordinates, full size);
    write() fills one (member, snapshot) slab of every state variable."""

    def __init__(self, filename, equation, lower, upper, dimension, num_samples, timesteps):
        self.filename = filename
        self.equation = equation
        self.dimension = tuple(int(d) for d in dimension)
        nx, ny, nz = self.dimension
        three = nz > 1
        self.cells = nx * ny * nz
        self.ntime = len(timesteps)
        self.num_samples = int(num_samples)
        dims = [("member", self.num_samples), ("time", self.ntime), ("x", nx), ("y", ny)]
        if three:
            dims.append(("z", nz))
        mids = cell_midpoints(lower, upper, self.dimension)
        coords = [("member", NC_INT, [0], np.arange(self.num_samples, dtype=">i4")),
                  ("time", NC_DOUBLE, [1], np.asarray(timesteps, dtype=">f8")),
                  ("x", NC_DOUBLE, [2], np.asarray(mids[0], dtype=">f8")),
                  ("y", NC_DOUBLE, [3], np.asarray(mids[1], dtype=">f8"))]
        if three:
            coords.append(("z", NC_DOUBLE, [4], np.asarray(mids[2], dtype=">f8")))
        state_dims = list(range(len(dims)))
        self.state = []
        for name, var in STATE_NAMES[equation]:
            if name == "mz" and not three:
                continue
            self.state.append((name, var))
        # header size first, then the offsets
        variables = [(n, t, d) for n, t, d, _ in coords] + [(n, NC_DOUBLE, state_dims) for n, _ in self.state]
        sizes = [a.nbytes for *_, a in coords] + [self.num_samples * self.ntime * self.cells * 8] * len(self.state)
        for s in sizes:
            if s >= 2 ** 32 - 4:
                raise ValueError("a NetCDF classic variable is limited to 4 GiB; use the numpy writer")
        header_len = len(self._header(dims, variables, sizes, [0] * len(variables)))
        begins, off = [], header_len
        for s in sizes:
            begins.append(off)
            off += s + (-s % 4)
        self.begins = dict(zip([v[0] for v in variables], begins))
        with open(filename, "wb") as f:
            f.write(self._header(dims, variables, sizes, begins))
            for (n, _, _, a), b in zip(coords, begins):
                f.seek(b)
                f.write(a.tobytes())
            f.truncate(off)

    @staticmethod
    def _header(dims, variables, sizes, begins):
        h = b"CDF\x02" + struct.pack(">i", 0)
        h += struct.pack(">ii", NC_DIMENSION, len(dims))
        for n, length in dims:
            h += _name(n) + struct.pack(">i", length)
        h += struct.pack(">ii", 0, 0)  # no global attributes
        h += struct.pack(">ii", NC_VARIABLE, len(variables))
        for (n, t, d), size, begin in zip(variables, sizes, begins):
            h += _name(n) + struct.pack(">i", len(d)) + b"".join(struct.pack(">i", i) for i in d)
            h += struct.pack(">ii", 0, 0)  # no variable attributes
            h += struct.pack(">ii", t, size + (-size % 4)) + struct.pack(">q", begin)
        return h

    def write(self, interior, member, snapshot, time=None):
        """interior: conserved variables (nvar, nz, ny, nx) of one sample at
        one save; member: the sample's index; snapshot: the save's index (the
        time coordinate is the file's save fraction, not `time`)."""
        if not (0 <= member < self.num_samples and 0 <= snapshot < self.ntime):
            raise IndexError("member %d / snapshot %d outside the file" % (member, snapshot))
        slab = (member * self.ntime + snapshot) * self.cells * 8
        with open(self.filename, "r+b") as f:
            for name, var in self.state:
                data = np.zeros(self.cells) if var is None else interior[var].reshape(-1)
                f.seek(self.begins[name] + slab)
                f.write(np.ascontiguousarray(data, dtype=">f8").tobytes())

    def finalize(self):
        pass


class NumpyWriter:
    """One .npz per snapshot: <basename>_<member>_<snapshot>.npz with the
    conserved variables by name (interior cells, arrays (nz, ny, nx)) and the
    time."""

    def __init__(self, basename, equation):
        self.basename = basename
        self.names = [n for n, _ in sorted(((n, v) for n, v in STATE_NAMES[equation] if v is not None),
                                            key=lambda p: p[1])]

    def write(self, interior, member, snapshot, time=None):
        path = "%s_%d_%d.npz" % (self.basename, member, snapshot)
        arrays = {n: interior[i] for i, n in enumerate(self.names)}
        if time is not None:
            arrays["time"] = np.array([time])
        np.savez(path, **arrays)

    def finalize(self):
        pass


def make_writer(writer_config, equation, lower, upper, dimension, num_samples, directory="."):
    """The fvm/stat writer of a configuration (WriterFactory::createWriter,
    alsfvm/src/io/WriterFactory.cpp:26-44)."""
    path = os.path.join(directory, writer_config.basename)
    if writer_config.type == "netcdf":
        return NetCDFWriter(path, equation, lower, upper, dimension, num_samples, writer_config.save_fractions())
    if writer_config.type == "numpy":
        return NumpyWriter(path, equation)
    raise ValueError("Unknown writer type %s" % writer_config.type)
