"""CPU model of how the OPM/FPGA Alveo kernel reads its packed input --
TEST INFRASTRUCTURE ONLY (the checker of gbilu_fpga_export).

Written from the kernel's RTL (paths under
linearalgebra/ilu0bicgstab/xilinx/src/rtl/bicgstab_solver_2r-3r3w/):
it reads the five data banks that fpga_copy_host_datamem fills (through the
byte offsets of the host library's layout) and runs the three operations the
kernel's sparstition unit runs on them:

* SpMV (sparstition.vhd:655-878, spmvp.vhd): for each color ("part") in
  order, its vector copy is gathered from the full vector through its P
  indices (int_read_unit.vhd: read_vect_inds); its values stream with their
  column indices into that copy and their new-row offsets, a value starting
  a new row iff its offset is non-zero and the offsets adding up to the row
  position, the row before the first being -1 (NR2offset.vhd:32-42); rows
  are written in order from the running row position (write_unit.vhd,
  arow rows per color);
* the L sweep (L_fs): the same with the partial results subtracted from the
  input p of the color's rows (ilu0.vhd: sub_res), the vector copy gathered
  from the results so far;
* the U sweep (U_bs): colors from the last, rows streaming in reverse
  (int_read_unit.vhd:296-299, ilu0.vhd:375-379); the differences of a block
  row's three scalar rows are aggregated in natural order and multiplied by
  the block diagonal, three values per scalar row (ilu0.vhd:360-362,
  ilu0.vhd:380-411: two multiplies added, then the third).

Per color the kernel reads the vector copy in 16-entry lines, the values in
8-value lines, the column indices in 32-index lines and the new-row offsets
in 64-offset lines (ext_read_unit.vhd:104,135,141), and the block diagonal
in 8-double lines (ext_read_unit.vhd:111-121), so every color's arrays start
on those boundaries. Layout offsets: gbilu_fpga_layout (the same as the
host library's, fpga_functions_bicgstab.cpp:176-305).
"""
from __future__ import annotations

import numpy as np


def up(v, m):
    return (v + m - 1) // m * m


# offsets[] order of gbilu_fpga_layout
OFF = dict(setup=0, nnz=(1, 2, 3), csize=(4, 5, 6), blkd=7, pidx=(8, 9, 10), cols=(11, 12, 13),
           nrs=(14, 15, 16))
BANK = dict(nnz=0, csize=0, blkd=0, pidx=1, cols=1, nrs=1)


class PackedSystem:
    """The kernel's view of a packed system: banks[5] (uint8 arrays),
    offsets[23] from gbilu_fpga_layout, processed_sizes[18]."""

    def __init__(self, banks, offsets, processed_sizes):
        self.banks = banks
        self.off = offsets
        self.ps = processed_sizes
        self.n = int(processed_sizes[0])

    def _arr(self, what, m, dtype, start, count):
        bank = self.banks[BANK[what]]
        o = int(self.off[OFF[what][m]]) + start * np.dtype(dtype).itemsize
        return np.frombuffer(bank, dtype, count, o)

    def parts(self, m):
        """(arow, col, val, pidx, vals, cols, nrs) per color of matrix m."""
        nc = int(self.ps[6 * m + 2])
        sizes = self._arr("csize", m, np.uint32, 0, 4 * nc).reshape(nc, 4)
        out = []
        p0 = v0 = c0 = r0 = 0
        for row, arow, col, val in sizes.astype(np.int64):
            pidx = self._arr("pidx", m, np.uint32, p0, col)
            vals = self._arr("nnz", m, np.float64, v0, val)
            cols = self._arr("cols", m, np.uint16, c0, val)
            nrs = self._arr("nrs", m, np.uint8, r0, val)
            out.append((int(arow), int(col), int(val), pidx.astype(np.int64), vals,
                        cols.astype(np.int64), nrs.astype(np.int64)))
            p0 += up(col, 16)
            v0 += up(val, 8)
            c0 += up(val, 32)
            r0 += up(val, 64)
        return out

    @staticmethod
    def _part_spmv(arow, col, vals, cols, nrs, vec, pidx):
        """Row sums of one color in stream order (rows never reached: 0)."""
        xp = vec[pidx]
        stream_row = np.cumsum(nrs) - 1
        if len(vals) and (stream_row.min() < 0 or stream_row.max() >= arow):
            raise ValueError("a new-row offset points outside the color")
        if len(cols) and cols.max() >= col:
            raise ValueError("a column index points outside the vector copy")
        acc = np.zeros(arow)
        np.add.at(acc, stream_row, vals * xp[cols])
        return acc

    def spmv(self, x):
        y = np.zeros(self.n)
        start = 0
        for arow, col, val, pidx, vals, cols, nrs in self.parts(0):
            y[start:start + arow] = self._part_spmv(arow, col, vals, cols, nrs, x, pidx)
            start += arow
        assert start == self.n
        return y

    def ilu_apply(self, p):
        y = np.array(p, dtype=np.float64)
        start = 0
        for arow, col, val, pidx, vals, cols, nrs in self.parts(1):
            s = self._part_spmv(arow, col, vals, cols, nrs, y, pidx)
            y[start:start + arow] = p[start:start + arow] - s
            start += arow
        assert start == self.n
        z = np.zeros(self.n)
        top = self.n
        d0 = 0
        blkd = np.frombuffer(self.banks[0], np.float64, int(self.ps[5]), int(self.off[OFF["blkd"]]))
        for arow, col, val, pidx, vals, cols, nrs in self.parts(2):
            s = self._part_spmv(arow, col, vals, cols, nrs, z, pidx)
            rows = np.arange(top - 1, top - 1 - arow, -1)          # stream order
            sub = y[rows] - s
            diag = blkd[d0:d0 + 4 * arow].reshape(arow, 4)[:, :3]
            for t in range(0, arow, 3):
                # stream rows 3i+2, 3i+1, 3i: aggregated in natural order
                a = sub[t:t + 3][::-1]
                blk_rows = rows[t:t + 3][::-1]
                for r in range(3):
                    d = diag[t + r]
                    z[blk_rows[r]] = (d[0] * a[0] + d[1] * a[1]) + d[2] * a[2]
            d0 += up(4 * arow, 8)
            top -= arow
        assert top == 0
        return z
