"""Copy the reference's real GOLDSTEIN masks into this fixture directory.

worbe2 (36x36, 8 levels) and worjh2 (36x36, 16 levels): the bathymetry (.k1, rows
j = maxj+1..0 of k1(0:maxi+1, j), land codes 18 and 90-99), the psi-point landmass labels
(.psiles, rows j = maxj..0) and the island path (.paths) that initialise_goldstein reads
(src/goldstein/goldstein.f90:1107-1123, 1502-1573).  Data files of the reference repository
(data/goldstein/), copied unchanged; tests read them through cgenie_gb300.grid.read_k1,
read_psiles and read_paths.

    python tests/golden/masks/make_golden_masks.py /path/to/cgenie
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ["worbe2", "worjh2"]


def main(ref_root: str) -> None:
    src = os.path.join(ref_root, "data", "goldstein")
    for n in NAMES:
        for ext in (".k1", ".psiles", ".paths"):
            shutil.copyfile(os.path.join(src, n + ext), os.path.join(HERE, n + ext))
            print("copied", n + ext)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
