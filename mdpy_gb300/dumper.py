"""Dumpers with mdpy's interface (mdpy/dumper/*.py).

``LogDumper`` lives in :mod:`mdpy_gb300.simulation`.  ``PDBDumper`` writes
one MODEL per dump (mdpy/dumper/pdb_dumper.py:14-27): the positions come
off the device in one copy and a writer thread formats and appends the
frame while the simulation continues on the GPU; ``flush()`` waits for the
frames in flight (``close()`` also ends the thread).  Records follow the
PDB format's fixed columns (CRYST1, MODEL, ATOM, ENDMDL).
"""
from __future__ import annotations

import queue
import threading

import numpy as np

from .error import FileFormatError
from .simulation import Dumper, LogDumper  # noqa: F401  (re-exported)


class PDBDumper(Dumper):
    def __init__(self, file_path: str, dump_frequency: int):
        if not str(file_path).endswith("pdb"):
            raise FileFormatError("The file should end with .pdb suffix")
        super().__init__(dump_frequency)
        self.file_path = str(file_path)
        open(self.file_path, "w").close()
        self._num_dumpped_frames = 0
        self._prefix = None
        self._queue = queue.Queue(maxsize=4)
        self._error = None
        self._thread = threading.Thread(target=self._writer, daemon=True)
        self._thread.start()

    # -- record layout ----------------------------------------------------------
    @staticmethod
    def _atom_prefixes(topology):
        n = topology.num_particles
        parts = getattr(topology, "particles", None) or []
        types = list(topology.particle_types)
        out = []
        for i in range(n):
            p = parts[i] if i < len(parts) else None
            name = (getattr(p, "particle_name", "") or types[i] or "X")[:4]
            res = (getattr(p, "molecule_type", None) or "MOL")[:3]
            chain = (getattr(p, "chain_id", None) or "A")[:1]
            resseq = getattr(p, "molecule_id", None)
            resseq = (i + 1) if resseq is None else int(resseq)
            out.append("ATOM  %5d %-4s %-3s %1s%4d    " % ((i + 1) % 100000, name, res, chain,
                                                          resseq % 10000))
        elements = ["%2s" % ((types[i] or "X")[:1]) for i in range(n)]
        return out, elements

    def _writer(self):
        while True:
            item = self._queue.get()
            if item is None:
                self._queue.task_done()
                return
            try:
                header, model, x = item
                lines = [header] if header else []
                lines.append("MODEL     %4d\n" % model)
                for pre, el, (a, b, c) in zip(self._prefix, self._elements, x):
                    lines.append("%s%8.3f%8.3f%8.3f%6.2f%6.2f          %s\n"
                                 % (pre, a, b, c, 1.0, 0.0, el))
                lines.append("ENDMDL\n")
                with open(self.file_path, "a") as fh:
                    fh.write("".join(lines))
            except Exception as exc:  # reported by flush()
                self._error = exc
            finally:
                self._queue.task_done()

    def dump(self, simulation):
        ens = simulation.ensemble
        header = None
        if self._num_dumpped_frames == 0:
            self._prefix, self._elements = self._atom_prefixes(ens.topology)
            box = np.diag(np.asarray(ens.state.pbc_matrix))
            header = "CRYST1%9.3f%9.3f%9.3f%7.2f%7.2f%7.2f\n" % (box[0], box[1], box[2],
                                                                90.0, 90.0, 90.0)
        x = ens.state.positions        # one device -> host copy
        self._num_dumpped_frames += 1
        self._queue.put((header, self._num_dumpped_frames, x))

    def flush(self):
        self._queue.join()
        if self._error is not None:
            raise self._error

    def close(self):
        if self._thread.is_alive():
            self._queue.put(None)
            self._thread.join()
        if self._error is not None:
            raise self._error

    @property
    def num_dumpped_frames(self):
        return self._num_dumpped_frames
