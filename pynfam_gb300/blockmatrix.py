"""Block-sparse matrices with one non-zero block per block row.

This is the data layout of the reference's ``blockmatrix`` type
(pnfam_type_blockmatrix.f90:22-26): block row ``i`` holds at most one block,
in block column ``cols[i]`` (``ir2c``), and the flat storage lists the blocks
in increasing block-row order, each block column-major (Fortran order).
The flat layout is what crosses the C ABI and what lives in device memory.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class BlockMatrix:
    cols: np.ndarray          # [nb] block column of each block row, -1 if empty
    blocks: list              # [nb] 2-D float64 arrays (db[i] x db[cols[i]]) or None

    @staticmethod
    def empty(cols, db) -> "BlockMatrix":
        cols = np.asarray(cols, dtype=np.int64)
        blocks = [None if c < 0 else np.zeros((int(db[i]), int(db[c]))) for i, c in enumerate(cols)]
        return BlockMatrix(cols, blocks)

    def offsets(self) -> np.ndarray:
        """Start of each block in the flat storage (``ir2m`` - 1); -1 if empty."""
        off = np.full(len(self.cols), -1, dtype=np.int64)
        p = 0
        for i, b in enumerate(self.blocks):
            if b is not None:
                off[i] = p
                p += b.size
        return off

    @property
    def nelem(self) -> int:
        return int(sum(b.size for b in self.blocks if b is not None))

    def flatten(self) -> np.ndarray:
        parts = [b.reshape(-1, order="F") for b in self.blocks if b is not None]
        return np.concatenate(parts) if parts else np.zeros(0)

    def set_flat(self, flat: np.ndarray) -> "BlockMatrix":
        p = 0
        for i, b in enumerate(self.blocks):
            if b is not None:
                n = b.size
                self.blocks[i] = np.asarray(flat[p:p + n], dtype=np.float64).reshape(b.shape, order="F").copy()
                p += n
        return self

    def copy(self) -> "BlockMatrix":
        return BlockMatrix(self.cols.copy(), [None if b is None else b.copy() for b in self.blocks])

    def to_dense(self, db) -> np.ndarray:
        db = np.asarray(db)
        st = np.concatenate([[0], np.cumsum(db)[:-1]])
        n = int(db.sum())
        d = np.zeros((n, n))
        for i, c in enumerate(self.cols):
            if c >= 0:
                d[st[i]:st[i] + db[i], st[c]:st[c] + db[c]] = self.blocks[i]
        return d
