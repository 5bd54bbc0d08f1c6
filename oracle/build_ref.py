"""TEST INFRASTRUCTURE ONLY — builds the reference's own CUDA kernels for golden fixtures.

Compiles the reference voxelproj extension (``voxelproj._CU``: the files
``voxelproj.cpp`` and ``projectors.cu`` with their ``include/*.cuh``) from the
source directory where they lie, with the reference's own nvcc flags
(``-O3 --use_fast_math``, setup.py:19-33) plus an sm_103a target, into
``oracle/_ref/`` (git-ignored).  The reference's setup.py is not run; this
recipe calls torch's extension builder on the two source files directly.

Only ``tests/golden/make_golden.py`` uses the result, to record the
reference's outputs as golden fixtures.  The voxelproj_gb300 package never
loads it.

    python oracle/build_ref.py --src DIR
    VOXELPROJ_REF_SRC=DIR python oracle/build_ref.py

DIR is the reference's ``voxelproj/csrc`` directory (``voxelproj.cpp``,
``projectors.cu`` and ``include/``), given by ``--src`` or else by the
environment variable ``VOXELPROJ_REF_SRC``.
"""

from __future__ import annotations

import argparse
import os
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SRC_ENV = "VOXELPROJ_REF_SRC"


def source_dir(src: Path | str | None = None) -> Path:
    """The reference's csrc directory: `src`, else $VOXELPROJ_REF_SRC."""
    if src:
        return Path(src)
    env = os.environ.get(SRC_ENV)
    if not env:
        raise FileNotFoundError(f"give the reference's voxelproj/csrc directory with --src or "
                                f"${SRC_ENV}")
    return Path(env)


def build(src: Path | None = None, verbose: bool = False):
    """Builds (or reuses) the reference extension and returns the module."""
    from torch.utils import cpp_extension

    src = source_dir(src)
    files = [src / "voxelproj.cpp", src / "projectors.cu"]
    for f in files:
        if not f.exists():
            raise FileNotFoundError(f"reference source {f} not found")
    OUT.mkdir(parents=True, exist_ok=True)
    # An explicit -gencode makes torch add no arch flags of its own.
    return cpp_extension.load(
        name="_CU",
        sources=[str(f) for f in files],
        extra_cflags=["-O3"],
        extra_cuda_cflags=["-O3", "--use_fast_math", "-gencode", "arch=compute_103a,code=sm_103a"],
        build_directory=str(OUT),
        verbose=verbose,
    )


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--src", type=Path, default=None)
    ap.add_argument("-v", "--verbose", action="store_true")
    args = ap.parse_args()
    os.environ.setdefault("MAX_JOBS", str(os.cpu_count() or 4))
    mod = build(args.src, args.verbose)
    print(mod.__file__)


if __name__ == "__main__":
    main()
