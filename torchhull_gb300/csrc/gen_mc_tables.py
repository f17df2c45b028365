"""Derive this library's marching-cubes triangulation table.

The triangulation must be the same one torchhull uses, so that face sets match
triangle for triangle.  torchhull ships it as ``face_table[256][16]`` in
``src/torchhull/_C/src/marching_cubes_table.h:61`` (BSD-3 data that torchhull
took from pytorch3d), indexed by a cube code whose bit order is permuted by
``index_table`` (``:342``) and listing edges in its own numbering
(``edge_to_vertex_table`` ``:335``, ``edge_direction_table`` ``:340``).

This script re-indexes that table into the convention used by the kernels and
the oracle here:

* corner ``i`` of the cell with base ``g`` is ``g + (i & 1, i >> 1 & 1, i >> 2 & 1)``
  (the same corner order as torchhull's ``cube_vertex``);
* bit ``i`` of a cell code is set when the value at corner ``i`` is below the
  isolevel (no permutation);
* an edge is one byte: bits 0-2 hold its lower corner ``c``, bits 3-4 its axis
  ``a`` (0 = x, 1 = y, 2 = z); the upper corner is ``c | (1 << a)``.

Triangle order inside a cell and vertex order inside a triangle are kept, so
the soup this table emits is the same soup torchhull emits.

Usage (needs the reference tree, so it runs only where that tree exists):
    python gen_mc_tables.py <path/to/marching_cubes_table.h> <out.h>
The generated header is committed; the build does not run this script.
"""

from __future__ import annotations

import re
import sys
from pathlib import Path

LICENSE = """\
// The triangulation data below descends from pytorch3d's marching-cubes tables
// (via torchhull), distributed under the BSD 3-Clause license:
//
// Copyright (c) Meta Platforms, Inc. and affiliates. All rights reserved.
//
// Redistribution and use in source and binary forms, with or without modification,
// are permitted provided that the following conditions are met:
//
//  * Redistributions of source code must retain the above copyright notice, this
//    list of conditions and the following disclaimer.
//
//  * Redistributions in binary form must reproduce the above copyright notice,
//    this list of conditions and the following disclaimer in the documentation
//    and/or other materials provided with the distribution.
//
//  * Neither the name Meta nor the names of its contributors may be used to
//    endorse or promote products derived from this software without specific
//    prior written permission.
//
// THIS SOFTWARE IS PROVIDED BY THE COPYRIGHT HOLDERS AND CONTRIBUTORS "AS IS" AND
// ANY EXPRESS OR IMPLIED WARRANTIES, INCLUDING, BUT NOT LIMITED TO, THE IMPLIED
// WARRANTIES OF MERCHANTABILITY AND FITNESS FOR A PARTICULAR PURPOSE ARE
// DISCLAIMED. IN NO EVENT SHALL THE COPYRIGHT HOLDER OR CONTRIBUTORS BE LIABLE FOR
// ANY DIRECT, INDIRECT, INCIDENTAL, SPECIAL, EXEMPLARY, OR CONSEQUENTIAL DAMAGES
// (INCLUDING, BUT NOT LIMITED TO, PROCUREMENT OF SUBSTITUTE GOODS OR SERVICES;
// LOSS OF USE, DATA, OR PROFITS; OR BUSINESS INTERRUPTION) HOWEVER CAUSED AND ON
// ANY THEORY OF LIABILITY, WHETHER IN CONTRACT, STRICT LIABILITY, OR TORT
// (INCLUDING NEGLIGENCE OR OTHERWISE) ARISING IN ANY WAY OUT OF THE USE OF THIS
// SOFTWARE, EVEN IF ADVISED OF THE POSSIBILITY OF SUCH DAMAGE.
"""


def _array(text: str, name: str) -> list[int]:
    m = re.search(name + r"[^=]*=\s*\{(.*?)\};", text, re.S)
    if m is None:
        raise ValueError(f"table {name} not found")
    body = re.sub(r"//[^\n]*", "", m.group(1)).replace("X", "255")
    return [int(v) for v in re.findall(r"-?\d+", body)]


def derive(src_text: str) -> tuple[list[int], list[list[int]]]:
    faces = _array(src_text, "face_table")
    counts_ref = _array(src_text, "vertex_number_table")
    e2v = _array(src_text, "edge_to_vertex_table")
    edir = _array(src_text, "edge_direction_table")
    perm = _array(src_text, "index_table")
    assert len(faces) == 256 * 16 and len(counts_ref) == 256 and len(e2v) == 24
    assert len(edir) == 12 and sorted(perm) == list(range(8))

    edge_code = []
    for e in range(12):
        lo, hi = e2v[2 * e], e2v[2 * e + 1]
        axis = {1: 0, 2: 1, 4: 2}[edir[e]]
        assert hi == lo | (1 << axis) and not lo & (1 << axis), "edge must run from lower to upper corner"
        edge_code.append(lo | (axis << 3))

    counts: list[int] = []
    table: list[list[int]] = []
    for code in range(256):
        ref_code = 0
        for i in range(8):
            if code >> i & 1:
                ref_code |= 1 << perm[i]
        row = faces[16 * ref_code : 16 * ref_code + 16]
        n = row.index(255) if 255 in row else 16
        assert n == counts_ref[ref_code] and n % 3 == 0 and n <= 15
        edges = [edge_code[e] for e in row[:n]]
        # Every edge with a sign change carries exactly the vertices the table uses.
        crossing = set()
        for c in range(8):
            for a in range(3):
                if c >> a & 1:
                    continue
                u = c | (1 << a)
                if (code >> c & 1) != (code >> u & 1):
                    crossing.add(c | (a << 3))
        assert set(edges) == crossing, f"code {code}: table edges differ from sign-change edges"
        counts.append(n)
        table.append(edges)
    return counts, table


def render(counts: list[int], table: list[list[int]]) -> str:
    out = [LICENSE, "", "// Generated by gen_mc_tables.py; do not edit by hand.", "#pragma once", ""]
    out.append("// Number of soup vertices (3 per triangle) emitted for each cell code.")
    out.append("#define TH_MC_TRI_COUNT_INIT { \\")
    for r in range(0, 256, 32):
        out.append("    " + ", ".join(str(c) for c in counts[r : r + 32]) + ", \\")
    out.append("}")
    out.append("")
    out.append("// Edge bytes for each cell code, 15 slots, unused slots 0xFF.")
    out.append("#define TH_MC_TRI_EDGES_INIT { \\")
    for code in range(256):
        row = table[code] + [255] * (15 - len(table[code]))
        out.append("    { " + ", ".join(str(v) for v in row) + " }, \\")
    out.append("}")
    out.append("")
    return "\n".join(out)


def main() -> None:
    src = Path(sys.argv[1]).read_text()
    counts, table = derive(src)
    Path(sys.argv[2]).write_text(render(counts, table))


if __name__ == "__main__":
    main()
