"""Minimal stand-in for pgenlib's PgenReader over a PLINK1 .bed, used only to run the
reference's bin/slemm_gamma.py here when generating golden vectors.  read(i, buf) fills the
allele-1 counts of variant i for the sample subset (pgenlib's convention; a missing call is -9).
"""
import numpy as np


class PgenReader:
    def __init__(self, path, raw_sample_ct=None, sample_subset=None):
        self.path = path.decode() if isinstance(path, bytes) else path
        raw = np.fromfile(self.path, dtype=np.uint8)
        assert raw[:3].tolist() == [0x6C, 0x1B, 0x01]
        self.n = int(raw_sample_ct)
        self.nb = (self.n + 3) // 4
        self.rows = raw[3:].reshape(-1, self.nb)
        self.subset = None if sample_subset is None else np.asarray(sample_subset, dtype=np.int64)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False

    def read(self, i, buf):
        row = self.rows[i]
        sh = np.array([0, 2, 4, 6], dtype=np.uint8)
        codes = ((row[:, None] >> sh) & 3).reshape(-1)[: self.n]
        a1 = np.choose(codes, [2, -9, 1, 0]).astype(np.int8)   # 00→2 A1, 01→missing, 10→1, 11→0
        if self.subset is not None:
            a1 = a1[self.subset]
        buf[:] = a1

    def read_list(self, idx, buf):
        for r, i in enumerate(idx):
            self.read(int(i), buf[r])
