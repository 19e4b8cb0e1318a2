"""The merged-model files (mergeddata.npz + mergedidxs.npz) written by
plenvdb_gb300.lifecycle.save_merged: the reference's keys and FP16 rows
(vdb_compression.py:55-58), and the row ids rebuilt from the occupancy bits
in C order. Host only."""
import numpy as np
import torch


def test_merged_files_round_trip(tmp_path):
    from plenvdb_gb300 import lifecycle as LC
    rng = np.random.default_rng(0)
    R = (7, 5, 9)
    occ = rng.random(R) < 0.4
    n = int(occ.sum())
    index = np.zeros(R, np.int32)
    index[occ] = np.arange(1, n + 1, dtype=np.int32)
    den = np.concatenate([[0], rng.normal(size=n)]).astype(np.float16)
    col = np.concatenate([np.zeros((1, 12)), rng.normal(size=(n, 12))]).astype(np.float16)
    merged = {"index": torch.from_numpy(index), "den": torch.from_numpy(den),
              "col": torch.from_numpy(col), "N": n + 1}
    LC.save_merged(str(tmp_path), merged)
    z = np.load(tmp_path / "mergeddata.npz")
    assert sorted(z.files) == ["col", "den"]
    assert z["den"].dtype == np.float16 and z["col"].dtype == np.float16
    d, c, idx, N = LC.load_merged(str(tmp_path))
    assert N == n + 1 and d.dtype == np.float32 and c.size == (n + 1) * 12
    np.testing.assert_array_equal(idx, index)
    np.testing.assert_array_equal(d, den.astype(np.float32))
    np.testing.assert_array_equal(LC.load_merged_index(str(tmp_path / "mergedidxs.npz")), index)


def test_merged_index_of_an_empty_mask(tmp_path):
    from plenvdb_gb300 import lifecycle as LC
    R = (3, 4, 5)
    merged = {"index": torch.zeros(R, dtype=torch.int32),
              "den": torch.zeros(1, dtype=torch.float16),
              "col": torch.zeros(1, 12, dtype=torch.float16), "N": 1}
    LC.save_merged(str(tmp_path), merged)
    d, c, idx, N = LC.load_merged(str(tmp_path))
    assert N == 1 and not idx.any() and idx.shape == R
