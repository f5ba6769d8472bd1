#!/bin/sh
# Regenerate the golden vectors with the reference's float executable.
# MANTA_REF_EXE: path of a mantaflow 0.13 `manta` built with -DNUMPY=ON
# (float precision, OpenMP or TBB).  One thread => serial reductions.
set -e
here=$(cd "$(dirname "$0")" && pwd)
exe=${MANTA_REF_EXE:?set MANTA_REF_EXE to the reference manta executable}
cd "$here"
OMP_NUM_THREADS=1 MANTA_DISABLE_UI=1 "$exe" make_golden.py "$here"
