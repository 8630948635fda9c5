"""Copy the netCDF-written restart file that the reference ships into this fixture folder.

data/main/main_restart_0.nc of the reference is a CDF-1 file written by the netCDF library
with the scalar calendar variables ioffset, iyear, imonth, iday over a dimension nrecs = 1,
the same definitions outm_netcdf (src/goldstein/goldstein_data.f90:238-260) makes.  The tests
use it to pin the restart codec's header and integer encoding to the library's bytes.

Usage: python tests/golden/restart/make_golden_restart.py <reference checkout>
"""
import hashlib
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref: str) -> None:
    src = os.path.join(ref, "data", "main", "main_restart_0.nc")
    dst = os.path.join(HERE, "main_restart_0.nc")
    shutil.copyfile(src, dst)
    print(dst, os.path.getsize(dst), hashlib.sha256(open(dst, "rb").read()).hexdigest())


if __name__ == "__main__":
    main(sys.argv[1])
