"""Checkpoint and restart of a long (T) evaluation.

The reference's restartable driver (src/tce/ccsd_t/ccsd_t_restart.F:58-90,
195-256) stores, after each outer p4b tile, the energies so far and the
position in the tuple loop in the run-time database
(tce:ccsd_t_restart_begin, tce:restart_triples_table) and resumes from
there.  Here the weight-ordered tuple list is evaluated in fixed ranges;
after each range its (E[T], E(T)) pair is appended to a JSON-lines file and
flushed to disk.  A restarted run reads the file, skips the ranges already
recorded and sums every recorded pair with math.fsum.  Ranges are
deterministic (each GPU evaluation of a range gives the same bits), so an
interrupted-and-resumed run returns exactly the energies of an
uninterrupted one.
"""
from __future__ import annotations

import hashlib
import json
import math
import os
from pathlib import Path
from typing import Callable

import numpy as np

Runner = Callable[[np.ndarray], tuple[float, float]]


def list_digest(klist: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(klist, dtype=np.int64).tobytes()).hexdigest()[:32]


class CheckpointedRun:
    """Evaluate klist in ranges of `chunk` tuples with `runner`, recording
    each finished range in `path`."""

    def __init__(self, path: str | Path, klist: np.ndarray, chunk: int, runner: Runner):
        if chunk < 1:
            raise ValueError("chunk must be positive")
        self.path = Path(path)
        self.klist = np.ascontiguousarray(klist, dtype=np.int64).reshape(-1, 7)
        self.chunk = int(chunk)
        self.runner = runner
        self.digest = list_digest(self.klist)
        self.ranges = [(b, min(b + self.chunk, len(self.klist))) for b in range(0, len(self.klist), self.chunk)]

    def done(self) -> dict[tuple[int, int], tuple[float, float]]:
        """Ranges already recorded for this tuple list (other lists' lines are ignored)."""
        out: dict[tuple[int, int], tuple[float, float]] = {}
        if not self.path.exists():
            return out
        for line in self.path.read_text().splitlines():
            try:
                r = json.loads(line)
            except json.JSONDecodeError:
                continue  # a line cut by an interruption
            if r.get("list") != self.digest or r.get("chunk") != self.chunk:
                continue
            out[(int(r["begin"]), int(r["end"]))] = (float(r["E[T]"]), float(r["E(T)"]))
        return out

    def run(self) -> tuple[float, float]:
        done = self.done()
        self.path.parent.mkdir(parents=True, exist_ok=True)
        with open(self.path, "a") as fh:
            for b, e in self.ranges:
                if (b, e) in done:
                    continue
                e1, e2 = self.runner(self.klist[b:e])
                done[(b, e)] = (float(e1), float(e2))
                fh.write(json.dumps({"list": self.digest, "chunk": self.chunk, "begin": b, "end": e,
                                     "E[T]": float(e1), "E(T)": float(e2)}) + "\n")
                fh.flush()
                os.fsync(fh.fileno())
        pairs = [done[r] for r in self.ranges]
        return math.fsum(p[0] for p in pairs), math.fsum(p[1] for p in pairs)

    @property
    def progress(self) -> float:
        d = self.done()
        return sum(e - b for (b, e) in self.ranges if (b, e) in d) / max(len(self.klist), 1)
