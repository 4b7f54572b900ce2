"""Restatement of the reference driver's particle writer writeTovtk
(src/main.cpp:127-164).  TEST INFRASTRUCTURE ONLY: the checker of
vfmm_write_vtk in tests/.

The reference streams every value through std::ostream with default flags,
which formats a double as printf "%g" (six significant digits) and a size_t
as a decimal integer; Python's "%g" operator follows the same C rules."""
from __future__ import annotations

import numpy as np


def reference_vtk_ascii(bodies: np.ndarray) -> bytes:
    """The bytes writeTovtk (main.cpp:127-164) writes for `bodies`."""
    n = bodies.size
    out = ["# vtk DataFile Version 3.0\n", "vtk output\n", "ASCII\n", "DATASET POLYDATA\n",
           f"POINTS {n} double\n"]                                            # :130-134
    out += ["%g %g %g\n" % tuple(b["X"]) for b in bodies]                    # :135-137
    out.append(f"VERTICES {n} {2 * n}\n")                                    # :139
    out += [f"1 {i}\n" for i in range(n)]                                    # :140-142
    out.append(f"POINT_DATA {n}\n")                                          # :143
    out.append("VECTORS alpha double\n")                                     # :146
    out += ["%g %g %g\n" % tuple(b["alpha"]) for b in bodies]                # :147-149
    out.append("VECTORS velocity double\n")                                  # :152
    out += ["%g %g %g\n" % tuple(b["velocity"]) for b in bodies]             # :153-155
    out += ["SCALARS radius double\n", "LOOKUP_TABLE default\n"]            # :158-159
    out += ["%g\n" % b["radius"] for b in bodies]                            # :160-162
    return "".join(out).encode()
