"""Samples files in the reference's NPY format.

A samples file `name.npy` holds a float64 array of shape (N, d+1) — one row
per stored sample, the misfit in the last column — and `name.npy.pkl` a
pickled dict of attributes (write_index, last_written_sample, proposals,
acceptance_rate, ...).  The reference's reader (`hmclab/Samples.py:23-278`)
loads it as `np.load(...).T`, i.e. as (d+1, N); this module writes the same
layout and reads both its own files and the reference's.  HDF5 files are
handled only when h5py is importable.
"""
import os as _os
import pickle as _pickle
import struct as _struct

import numpy as _numpy

_HEADER_SPARE = 64


class _NpyAppender:
    """Growable .npy file: a version-2.0 header with spare room for the shape,
    rows appended at the end and the shape rewritten in place."""

    def __init__(self, filename, columns):
        self.filename = filename
        self.columns = int(columns)
        self.rows = 0
        self.fp = open(filename, "wb")
        self.header_len = len(self._header(0))
        self.fp.write(self._header(0))

    def _header(self, rows):
        d = {"descr": "<f8", "fortran_order": False, "shape": (rows, self.columns)}
        body = repr(d).encode("latin1")
        # magic(6) + version(2) + length(4) + body + padding + '\n', total % 64 == 0
        base = 6 + 2 + 4 + len(body) + 1
        total = ((base + _HEADER_SPARE + 63) // 64) * 64
        body = body + b" " * (total - base) + b"\n"
        return b"\x93NUMPY" + bytes([2, 0]) + _struct.pack("<I", len(body)) + body

    def append(self, rows_array):
        a = _numpy.ascontiguousarray(rows_array, dtype="<f8")
        assert a.ndim == 2 and a.shape[1] == self.columns
        self.fp.seek(0, 2)
        self.fp.write(a.tobytes())
        self.rows += a.shape[0]
        hdr = self._header(self.rows)
        assert len(hdr) == self.header_len
        self.fp.seek(0)
        self.fp.write(hdr)
        self.fp.flush()

    def close(self):
        if self.fp is not None:
            self.fp.close()
            self.fp = None


class Samples:
    """Read or write a samples file (reference `hmclab/Samples.py:16-412`)."""

    def __init__(self, filename, burn_in=None, mode="r", overwrite=None):
        stem, ext = _os.path.splitext(filename)
        if ext == "" or ext == ".h5":
            self.filetype = "HDF5"
            filename = stem + ".h5"
        elif ext == ".npy":
            self.filetype = "NPY"
        else:
            raise AttributeError(f"Unkown extension `{ext}` for samples file.")
        self.mode = mode
        self.filename = filename
        self._attrs = {}
        if mode == "r":
            if overwrite is not None:
                raise AttributeError("Overwrite is not relevant when writing samples.")
            if not _os.path.isfile(filename):
                raise FileNotFoundError(f"Trying to read samples file `{filename}` which does not exist.")
            if self.filetype == "HDF5":
                import h5py  # noqa: F401 - optional dependency

                self._h5 = h5py.File(filename, "r")
                self._array = self._h5["samples"]
                self._attrs = dict(self._array.attrs)
            else:
                self._array = _numpy.load(filename, mmap_mode="r").T
                with open(f"{filename}.pkl", "rb") as f:
                    self._attrs = _pickle.load(f)
            self.burn_in = 0 if burn_in is None else burn_in
            self.last_sample = self.read_attribute("write_index")
            if self.last_sample <= self.burn_in:
                raise ValueError(
                    "The burn-in phase is longer than the chain itself. "
                    f"Total samples before burn in: {self.last_sample}"
                )
        elif mode == "w":
            if burn_in is not None:
                raise AttributeError("Burn in is not relevant when writing samples.")
            directory = _os.path.dirname(filename)
            if directory != "" and not _os.path.isdir(directory):
                raise NotADirectoryError(f"Trying to write a samples file to a non-existent directory `{directory}`.")
            overwrite = bool(overwrite)
            if (not overwrite) and (
                _os.path.isfile(filename) or (self.filetype == "NPY" and _os.path.isfile(f"{filename}.pkl"))
            ):
                raise FileExistsError(f"Trying to write samples to an already existing file `{filename}`.")
            if self.filetype == "HDF5":
                raise NotImplementedError("HDF5 samples files need h5py; use a `.npy` filename")
            self._appender = None
            self.write_attribute("write_index", 0)
            self.write_attribute("last_written_sample", -1)
        else:
            raise AttributeError(f"Unkown file mode `{mode}` for samples file.")

    # ---- attributes -------------------------------------------------------
    def write_attribute(self, name, value):
        assert self.mode == "w"
        self._attrs[name] = value

    def read_attribute(self, name):
        return self._attrs[name]

    # ---- data -------------------------------------------------------------
    def append_columns(self, block):
        """Append samples given as columns: block is (d+1, n)."""
        assert self.mode == "w"
        block = _numpy.asarray(block, dtype=_numpy.float64)
        if self._appender is None:
            self._appender = _NpyAppender(self.filename, block.shape[0])
        self._appender.append(block.T)
        self._attrs["write_index"] += block.shape[1]
        self._attrs["last_written_sample"] += block.shape[1]

    append = append_columns

    @property
    def numpy(self):
        return self._array[:, self.burn_in :]

    def __getitem__(self, key):
        return self.numpy[key]

    def close(self):
        if self.mode == "w":
            if self._appender is None:
                # no samples: still leave a valid (0, 0) array behind
                _numpy.save(self.filename, _numpy.zeros((0, 0)))
            else:
                self._appender.close()
            with open(f"{self.filename}.pkl", "wb") as f:
                _pickle.dump(self._attrs, f)
        elif self.filetype == "HDF5":
            self._h5.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def combine_samples(filenames, output_filename=None, cores=None, overwrite_existing_file=False):
    """Stack the samples of several files along a chain axis: returns an array
    of shape (n_files, d+1, N_min) (reference `hmclab/Samples.py:415-456`
    returns the same chains concatenated; both are offered via the axis)."""
    arrays = []
    for fn in filenames:
        with Samples(fn) as s:
            arrays.append(_numpy.array(s.numpy))
    n = min(a.shape[1] for a in arrays)
    out = _numpy.stack([a[:, :n] for a in arrays], axis=0)
    if output_filename is not None:
        w = Samples(output_filename, mode="w", overwrite=overwrite_existing_file)
        w.append_columns(_numpy.hstack(list(out)))
        w.close()
    return out
