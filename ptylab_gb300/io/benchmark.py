"""Throughput of the measurement / result file path.

    python -m ptylab_gb300.io.benchmark [--frames 400 --Nd 128] [--reps 5]

Writes a synthetic CPM measurement file (float32 ptychogram of ``frames`` x
``Nd`` x ``Nd`` plus the scalar fields), once contiguous and once chunked
with gzip + shuffle, then times (best of ``reps``, page cache warm):

* ``write``: ``hdf5.File(.., "w")`` + ``create_dataset`` of all fields;
* ``load``: ``ExperimentalData(filename)``, the reference's entry point
  (field checks, reads, scalars, orientation, ``_setData``'s frame sums);
* ``read``: the ptychogram dataset alone;
* ``fromfile``: ``np.fromfile`` of the same bytes at the same offset, the
  bound any reader of a contiguous dataset meets;

and prints one JSON line per file layout, in MB/s of ptychogram bytes.
"""

from __future__ import annotations

import argparse
import json
import os
import tempfile
import time

import numpy as np

from ..ExperimentalData import ExperimentalData
from . import hdf5


def _best(fn, reps):
    best = float("inf")
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        best = min(best, time.perf_counter() - t0)
    return best


def _write(path, frames, enc, **opts):
    with hdf5.File(path, "w") as hf:
        hf.create_dataset("ptychogram", data=frames, dtype="f", **opts)
        hf.create_dataset("encoder", data=enc, dtype="f")
        hf.create_dataset("dxd", data=(7.2e-6,), dtype="f")
        hf.create_dataset("zo", data=(0.05,), dtype="f")
        hf.create_dataset("wavelength", data=(632.8e-9,), dtype="f")
        hf.create_dataset("orientation", data=0)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--frames", type=int, default=400)
    ap.add_argument("--Nd", type=int, default=128)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--dir", default=None, help="directory for the files (default: a temporary one)")
    args = ap.parse_args(argv)

    rng = np.random.default_rng(0)
    frames = rng.poisson(50.0, (args.frames, args.Nd, args.Nd)).astype(np.float32)
    enc = rng.standard_normal((args.frames, 2)).astype(np.float32) * 1e-5
    mb = frames.nbytes / 1e6
    with tempfile.TemporaryDirectory(dir=args.dir) as d:
        for layout, opts in (("contiguous", {}), ("gzip", dict(chunks=(1, args.Nd, args.Nd),
                                                                 compression="gzip", shuffle=True))):
            path = os.path.join(d, f"{layout}.hdf5")
            t_write = _best(lambda: _write(path, frames, enc, **opts), args.reps)
            t_load = _best(lambda: ExperimentalData(path), args.reps)

            def read():
                with hdf5.File(path) as f:
                    return f["ptychogram"][()]

            got = read()
            if not np.array_equal(got, frames):
                raise SystemExit(f"{layout}: read back differs from what was written")
            t_read = _best(read, args.reps)
            line = {
                "metric": "hdf5 measurement file throughput", "unit": "MB/s", "layout": layout,
                "frames": args.frames, "Nd": args.Nd, "ptychogram_MB": round(mb, 2),
                "file_MB": round(os.path.getsize(path) / 1e6, 2),
                "write": round(mb / t_write, 1), "load": round(mb / t_load, 1), "read": round(mb / t_read, 1),
            }
            if layout == "contiguous":
                with hdf5.File(path) as f:
                    r = f._reader
                    for m in r.messages(f._links["ptychogram"]):
                        if m.type == hdf5.MSG_LAYOUT:
                            addr = int.from_bytes(m.data[2:10], "little")
                off = r.base + addr

                def raw():
                    with open(path, "rb") as fh:
                        fh.seek(off)
                        return np.fromfile(fh, dtype=np.float32, count=frames.size)

                line["fromfile"] = round(mb / _best(raw, args.reps), 1)
            print(json.dumps(line))


if __name__ == "__main__":
    main()
