"""chopSuey, the brick preprocessing tool, for raw volumes.

    python -m aloha_gb300.chopsuey in.raw -dims X Y Z -type uint8|uint16|float -n N -o out.vol

Same command line and output as the reference tool's volume path
(chopSuey.cpp:361-441): the raw file (x fastest, no header) is memory-mapped,
split by the middle-split VolumeSplitter into N bricks (at least two, as the
tool gives for -n 1) with a one-voxel upper ghost layer, each brick
normalised like Volume::get (uint8 /255, uint16 /65535, float as is) with its
value range, and written as a .vol file.  ``-bpc 1|2|4`` selects the type by
bytes per voxel, as in the reference.  The reference's .obj (triangle mesh)
input is not part of this package: it exits with status 1.
"""
from __future__ import annotations

import sys

from . import volfile


def usage(err: str) -> int:
    if err:
        sys.stderr.write(f"\nFatal error: {err}\n\n")
    sys.stderr.write("Usage: python -m aloha_gb300.chopsuey in.raw -dims x y z -type uint8|uint16|float "
                     "-n numBricks -o out.vol\n")
    return 1


def main(argv=None) -> int:
    argv = list(sys.argv[1:] if argv is None else argv)
    in_file, out_file, n, dims, bpc = "", "chopSuey.tri", 1, (0, 0, 0), 1
    i = 0
    try:
        while i < len(argv):
            arg = argv[i]
            if not arg.startswith("-"):
                in_file = arg
            elif arg == "-o":
                i += 1
                out_file = argv[i]
            elif arg == "-n":
                i += 1
                n = int(argv[i])
            elif arg == "-dims":
                dims = (int(argv[i + 1]), int(argv[i + 2]), int(argv[i + 3]))
                i += 3
            elif arg == "-bpc":
                i += 1
                bpc = int(argv[i])
            elif arg == "-type":
                i += 1
                t = argv[i]
                if t not in ("uint8", "uint16", "float"):
                    return usage(f"wrong type '{t}'")
                bpc = {"uint8": 1, "uint16": 2, "float": 4}[t]
            else:
                return usage(f"unknown cmdline arg '{arg}'")
            i += 1
    except (IndexError, ValueError):
        return usage(f"missing or bad value for '{argv[i] if i < len(argv) else argv[-1]}'")
    if not in_file:
        return usage("no filename specified")
    if not in_file.endswith(".raw"):
        return usage("only .raw volumes are supported (triangle meshes are not part of this package)")
    if dims == (0, 0, 0):
        return usage("no input dimensions specified")
    if bpc not in volfile.BPC_TYPES:
        return usage("no data type/bpc specified")
    try:
        descs = volfile.chop_raw(in_file, dims, volfile.BPC_TYPES[bpc], n, out_file)
    except (OSError, ValueError) as e:
        return usage(str(e))
    for d in descs:
        print(d["cell_lo"], d["cell_hi"], d["voxel_lo"], d["voxel_hi"], d["value_range"])
    return 0


if __name__ == "__main__":
    sys.exit(main())
