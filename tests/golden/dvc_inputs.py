"""Input files of the end-to-end `dvc` runs: raw volumes (fixed-length
header, byte order), point cloud and keyword input file, written from the
fixture volumes. Shared by make_golden.py (which runs the reference's `dvc` on
them) and tests/test_host_programs.py (which runs the drop-in `dvc`)."""
from __future__ import annotations

import os

import numpy as np


def write_dvc_inputs(d, case, vols, pts, labels):
    vref, vcor = vols[case["volumes"]]
    bits = 8 * vref.dtype.itemsize
    for name, v in (("ref.raw", vref), ("cor.raw", vcor)):
        a = v.astype(">u2") if (bits == 16 and case["endian"] == "big") else v
        with open(os.path.join(d, name), "wb") as f:
            f.write(bytes(i % 256 for i in range(case["header"])))
            f.write(np.ascontiguousarray(a).tobytes())
    with open(os.path.join(d, "points.roi"), "w") as f:
        f.write(case["roi_extra"])
        for lab, p in zip(labels, pts):
            f.write(f"{lab}\t{p[0]:g}\t{p[1]:g}\t{p[2]:g}\n")
    z, y, x = vref.shape
    lines = ["# drop-in test run", "reference_filename\tref.raw\t### reference",
             "correlate_filename\tcor.raw\t### correlate", "point_cloud_filename\tpoints.roi\t###",
             "output_filename\tresult\t###", f"vol_bit_depth\t{bits}\t###"]
    if bits == 16:
        lines.append(f"vol_endian\t{case['endian']}\t###")
    lines += [f"vol_hdr_lngth\t{case['header']}\t###", f"vol_wide\t{x}\t###",
              f"vol_high\t{y}\t###", f"vol_tall\t{z}\t###"]
    lines += [f"{k}\t{v}\t### setting" for k, v in case["keys"]]
    with open(os.path.join(d, "dvc_in"), "w") as f:
        f.write("\n".join(lines) + "\n")
