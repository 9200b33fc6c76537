"""Pack the EDKnrc energy-deposition-kernel listings into one compact .npz.

The engine needs the 48-cone x 24-sphere ``total`` column of each of the
twelve monoenergetic EDKnrc runs that ship with conehead
(``kernels/<E>MeV/<E>MeV.egslst``).  This script parses those listings the
same way ``conehead/kernel.py:27-45`` does (rows between the
"angle/deg.  radius/cm" header + 2 and "END OF RUN" - 1, first three
columns as float32) and stores, per energy label, the raw (1152, 3) float32
block plus the kinetic energy quoted in the listing.

Usage::

    python conehead_gb300/data/extract_edknrc.py <conehead checkout> [out.npz]

The packaged ``edknrc_6mv.npz`` next to this file was produced by running it
on the conehead sources.  ``KernelMono`` can also read ``.egslst`` files
directly, so the .npz is a convenience, not a second format.
"""
import os
import sys

import numpy as np

LABELS = ["0.5", "1.0", "1.5", "2.0", "2.5", "3.0",
          "3.5", "4.0", "4.5", "5.0", "5.5", "6.0"]


def parse_egslst(path):
    """Return (energy_MeV, data_raw float32 [n, 3]) from one .egslst file."""
    with open(path) as f:
        lines = f.readlines()
    energy = None
    start = end = None
    for i, line in enumerate(lines):
        if "KINETIC ENERGY OF THE INCIDENT BEAM:" in line:
            energy = float(line.split()[-2])
        if "angle/deg.  radius/cm" in line:
            start = i + 2
        if "END OF RUN" in line:
            end = i - 1
    if start is None or end is None:
        raise ValueError(f"{path}: kernel table markers not found")
    rows = [ln.split()[:3] for ln in lines[start:end]]
    return energy, np.array(rows, dtype=np.float32)


def main(argv):
    if len(argv) < 2:
        print(__doc__)
        return 2
    root = argv[1]
    out = argv[2] if len(argv) > 2 else os.path.join(
        os.path.dirname(os.path.abspath(__file__)), "edknrc_6mv.npz")
    payload = {}
    for lab in LABELS:
        path = os.path.join(root, "kernels", f"{lab}MeV", f"{lab}MeV.egslst")
        energy, data = parse_egslst(path)
        if data.shape != (1152, 3):
            raise ValueError(f"{path}: expected 1152 rows, got {data.shape}")
        payload[f"E{lab}"] = data
        payload[f"energy_{lab}"] = np.float64(energy)
    np.savez_compressed(out, **payload)
    print(f"wrote {out}")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
