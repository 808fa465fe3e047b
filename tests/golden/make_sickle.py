"""Fixture of the reference's sample sickle cell (sample_files/sample_cells/
SickleCell.dat of the RBC3D tree: nlat0 12, a 36 x 72 Gauss grid), read with
the ImportReadRBC restatement of rbc3d_gb300.state_io and saved as
sickle_cell.npz (positions as ImportReadRBC leaves them, recentred).

    python tests/golden/make_sickle.py /path/to/RBC3D/sample_files/sample_cells/SickleCell.dat
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from rbc3d_gb300 import state_io  # noqa: E402


def main(src):
    c = state_io.import_read_rbc(src)
    np.savez_compressed(os.path.join(HERE, "sickle_cell.npz"), nlat0=c.nlat0, nlon0=c.nlon0, nlat=c.nlat,
                        nlon=c.nlon, celltype=c.celltype, x=c.x)
    print(f"nlat0 {c.nlat0} nlon0 {c.nlon0} grid {c.nlat} x {c.nlon} celltype {c.celltype}")


if __name__ == "__main__":
    main(sys.argv[1])
