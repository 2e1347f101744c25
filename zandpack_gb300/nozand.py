"""``nozand`` on one GPU: ``python -m zandpack_gb300.nozand Dir=/path/to/run``.

Drop-in for ``mpirun -np P nozand Dir=...`` (Zandpack/mpi/nozand): the
``zand`` run directory plus ``Arrays/S^(-0.5)``, propagated in the
non-orthogonal basis (``zandpack_gb300.zand.ZandRun`` with ``nonorth=True``).
"""
from __future__ import annotations

import sys

from .zand import ZandRun, parse_dir


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    ZandRun(parse_dir(argv), nonorth=True).run()


if __name__ == "__main__":
    main()
