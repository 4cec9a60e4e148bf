"""Command-line runner with the run-process's arguments:

    python -m svl_gb300.run -dir /path/to/Partition/ -file 'Model.1.$.json' [more files]

The file is a partition written by the pre-processor; `$` stands for the
process rank (RP/12-Utilities/Driver.hpp:255-265), 0 here: one GPU runs one
partition, with its integrator, algorithm and recorders; node recorders go
to `<dir>/../Solution/<combination>/` as the run-process writes them
(RP/12-Utilities/Recorder.cpp:73-106).  Exit status 0 on success, 1 when a
step fails ("A PROBLEM WAS ENCOUNTERED"), 2 for bad arguments or files.

One file per run.  The run-process's RunDriverFile (Driver.hpp:2049-2101)
treats several -file arguments as consecutive stages on ONE mesh: later
files add, delete or modify entities of it and continue from the previous
stage's displacements and material states.  Those stage updates are not
covered here, so more than one file is rejected (status 2) rather than run
from rest on a fresh model, which would give different results."""
from __future__ import annotations

import sys
import time
from pathlib import Path
from typing import List, Optional, Tuple

from .partition import Partition, PartitionError, load_partition


def parse_args(argv: List[str]) -> Tuple[Optional[Path], List[str]]:
    """-dir and -file as CommandLine reads them (RP/12-Utilities/Utilities.hpp:
    97-160): -file takes every following argument up to the next flag."""
    path, files = None, []
    i = 0
    while i < len(argv):
        a = argv[i].lower()
        if a == "-dir" and i + 1 < len(argv):
            path = Path(argv[i + 1])
            i += 2
        elif a == "-file":
            i += 1
            while i < len(argv) and argv[i].lower() not in ("-dir", "--h", "--help"):
                files.append(argv[i])
                i += 1
        else:
            i += 1
    return path, files


def resolve(path: Path, names: List[str], rank: int = 0) -> List[Path]:
    """The partition files of this rank: `$` replaced by the rank."""
    return [path / n.replace("$", str(rank)) for n in names]


def load_all(path: Path, names: List[str]) -> List[Partition]:
    out = []
    for f in resolve(path, names):
        if not f.is_file():
            raise PartitionError("The JSON file '%s' couldn't be opened." % f)
        out.append(load_partition(f))
    return out


def main(argv: Optional[List[str]] = None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    if any(a.lower() in ("--h", "--help") for a in argv) or not argv:
        print(__doc__)
        return 0 if argv else 2
    path, names = parse_args(argv)
    if path is None or not names:
        print("ERROR: NOT ENOUGH Command line input arguments (-dir and -file).")
        return 2
    if len(names) > 1:
        print("ERROR: %d files given; staged runs (several -file arguments continuing on one mesh) are not "
              "covered, run one partition file per call." % len(names))
        return 2
    try:
        parts = load_all(path, names)
    except (PartitionError, ValueError, KeyError) as exc:
        print("ERROR: %s" % exc)
        return 2
    for p in parts:
        t0 = time.perf_counter()
        try:
            p.run(write_recorders=True)
        except (RuntimeError, PartitionError) as exc:
            print("A PROBLEM WAS ENCOUNTERED: %s" % exc)
            return 1
        print("Analysis %s (%s, %d steps) finished in %.3f s" % (p.combo_folder, p.integrator, p.nt - 1,
                                                                 time.perf_counter() - t0))
    return 0


if __name__ == "__main__":
    sys.exit(main())
