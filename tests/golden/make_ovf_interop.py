"""Writes the OVF interoperability fixtures in tests/golden/ovf_interop/.

    python tests/golden/make_ovf_interop.py

Each file holds the same 4 x 3 x 2 vector field, laid out as the OOMMF OVF
format documents describe (OVF 2.0 and OVF 1.0 rectangular meshes) in the
variants other micromagnetic codes write:

- ovf2_b4_desc.ovf: OVF 2.0, "Data Binary 4" (little-endian, check value
  1234567.0), reduced m, the header keys in the order Title, meshtype,
  meshunit, x/y/zmin, x/y/zmax, valuedim, valuelabels, valueunits, Desc,
  x/y/zbase, x/y/znodes, x/y/zstepsize (the layout GPU finite-difference codes
  such as mumax3 use);
- ovf2_b8_comments.ovf: OVF 2.0, "Data Binary 8" (check value
  123456789012345.0), the magnetisation M = Ms m in A/m, "##" comment lines,
  several Desc lines, lower-case "data binary 8" (as OOMMF's own writers may);
- ovf1_b4_bigendian.omf: OVF 1.0 ("# OOMMF: rectangular mesh v1.0"),
  big-endian Binary 4 with valuemultiplier 800000, boundary-xyz and
  ValueRange keys: the stored numbers times the multiplier are M in A/m;
- ovf2_text_spacing.ovf: OVF 2.0 "Data Text" with irregular spacing and a
  comment line inside the data.

field(): the values (x fastest, then y, then z), unit vectors m; MS scales
them to A/m where a file stores M.
"""
import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "ovf_interop")
NX, NY, NZ = 4, 3, 2
DX, DY, DZ = 2e-9, 1.5e-9, 1e-9
MS = 8e5


def field():
    """(3, n) unit vectors, x fastest."""
    n = NX * NY * NZ
    i = np.arange(n)
    th = 0.3 + 0.11 * i
    ph = 0.7 * i
    return np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)])


def _geom_lines():
    return [f"# xbase: {DX / 2!r}", f"# ybase: {DY / 2!r}", f"# zbase: {DZ / 2!r}",
            f"# xnodes: {NX}", f"# ynodes: {NY}", f"# znodes: {NZ}",
            f"# xstepsize: {DX!r}", f"# ystepsize: {DY!r}", f"# zstepsize: {DZ!r}"]


def _extent_lines():
    return ["# xmin: 0", "# ymin: 0", "# zmin: 0", f"# xmax: {NX * DX!r}", f"# ymax: {NY * DY!r}",
            f"# zmax: {NZ * DZ!r}"]


def write_ovf2_b4(path):
    v = field().T.astype("<f4")
    head = (["# OOMMF OVF 2.0", "# Segment count: 1", "# Begin: Segment", "# Begin: Header", "# Title: m",
             "# meshtype: rectangular", "# meshunit: m"] + _extent_lines()
            + ["# valuedim: 3", "# valuelabels: m_x m_y m_z", "# valueunits: 1 1 1",
               "# Desc: Total simulation time:  0  s"] + _geom_lines() + ["# End: Header", "# Begin: Data Binary 4"])
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode())
        f.write(struct.pack("<f", 1234567.0))
        f.write(v.tobytes())
        f.write(b"\n# End: Data Binary 4\n# End: Segment\n")


def write_ovf2_b8(path):
    v = (MS * field()).T.astype("<f8")
    head = (["# OOMMF OVF 2.0", "#", "# Segment count: 1", "#", "# Begin: Segment", "# Begin: Header", "#",
             "# Title: Oxs_TimeDriver::Magnetization", "# Desc: Iteration: 120, Phase: 1",
             "# Desc: Stage: 0, Stage iteration: 120", "## a comment line with a colon: ignored",
             "# meshtype: rectangular", "# meshunit: m"] + _extent_lines()
            + ["# valuedim: 3", "# valuelabels: Magnetization_x Magnetization_y Magnetization_z",
               "# valueunits: A/m A/m A/m", "#"] + _geom_lines() + ["#", "# End: Header", "#",
                                                                    "# Begin: data binary 8"])
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode())
        f.write(struct.pack("<d", 123456789012345.0))
        f.write(v.tobytes())
        f.write(b"\n# End: data binary 8\n# End: segment\n")


def write_ovf1_b4_be(path):
    v = field().T.astype(">f4")  # stored values; times valuemultiplier = M in A/m
    head = (["# OOMMF: rectangular mesh v1.0", "# Segment count: 1", "# Begin: Segment", "# Begin: Header",
             "# Title: m", "# Desc: OVF 1.0 with a value multiplier", "# meshunit: m", "# valueunit: A/m",
             f"# valuemultiplier: {MS!r}"] + _extent_lines()
            + ["# ValueRangeMaxMag: 1.0", "# ValueRangeMinMag: 1e-8", "# meshtype: rectangular"]
            + _geom_lines() + [f"# boundary-xyz: 0 0 0 {NX * DX!r} 0 0 {NX * DX!r} {NY * DY!r} 0",
                               "# End: Header", "# Begin: Data Binary 4"])
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode())
        f.write(struct.pack(">f", 1234567.0))
        f.write(v.tobytes())
        f.write(b"\n# End: Data Binary 4\n# End: Segment\n")


def write_ovf2_text(path):
    v = field().T
    head = (["# OOMMF OVF 2.0", "# Segment count: 1", "# Begin: Segment", "# Begin: Header", "# Title: m",
             "# meshtype: rectangular", "# meshunit: m", "# valuedim: 3", "# valuelabels: m_x m_y m_z",
             "# valueunits: 1 1 1"] + _geom_lines() + ["# End: Header", "# Begin: Data Text"])
    lines = []
    for k, row in enumerate(v):
        if k == NX * NY:
            lines.append("# next layer")
        lines.append("  " + "   ".join(repr(float(x)) for x in row))
    with open(path, "w") as f:
        f.write("\n".join(head + lines) + "\n# End: Data Text\n# End: Segment\n")


FILES = {"ovf2_b4_desc.ovf": write_ovf2_b4, "ovf2_b8_comments.ovf": write_ovf2_b8,
         "ovf1_b4_bigendian.omf": write_ovf1_b4_be, "ovf2_text_spacing.ovf": write_ovf2_text}

if __name__ == "__main__":
    os.makedirs(OUT, exist_ok=True)
    for name, fn in FILES.items():
        fn(os.path.join(OUT, name))
        print("wrote", name, os.path.getsize(os.path.join(OUT, name)), "bytes")
