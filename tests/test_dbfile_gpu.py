"""Database file (tsim_db_save / tsim_db_load): a loaded database answers
exactly like the one it was written from; damaged files are refused."""
import numpy as np
import pytest

from cudaruntime1_gb300 import datagen as G

pytestmark = pytest.mark.gpu


def test_database_file_round_trip(tsim, cuda_ctx, tmp_path):
    """tsim_db_save / tsim_db_load: the loaded database answers exactly like
    the one it was written from; damaged files are refused."""
    cp, co = G.random_walks(1500, G.uniform_lengths(1500, 8, 200, 8), 9)
    qp, qo = G.random_walks(12, G.uniform_lengths(12, 8, 200, 10), 11)
    db = tsim.Database(cuda_ctx, cp, co)
    path = tmp_path / "db.tsim"
    db.save(path)
    db2 = tsim.Database(cuda_ctx, path=path)
    assert db2.count == db.count and db2.device_bytes() == db.device_bytes()
    for measure, kw in [("dtw", dict(band_pct=10)), ("lcss", dict(epsilon=0.5, delta=10)),
                        ("frechet", {}), ("hausdorff", {}), ("euclidean", {})]:
        a = tsim.knn(cuda_ctx, db, qp, qo, measure, 10, stats=False, **kw)
        b = tsim.knn(cuda_ctx, db2, qp, qo, measure, 10, stats=False, **kw)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), measure
    raw = bytearray(path.read_bytes())
    bad = tmp_path / "flipped.tsim"
    raw[len(raw) // 2] ^= 0x40
    bad.write_bytes(bytes(raw))
    with pytest.raises(tsim.api._lib.TsimError):
        tsim.Database(cuda_ctx, path=bad)
    short = tmp_path / "short.tsim"
    short.write_bytes(path.read_bytes()[:-100])
    with pytest.raises(tsim.api._lib.TsimError):
        tsim.Database(cuda_ctx, path=short)
    # a header claiming 2^31 - 1 trajectories is refused by its size, before
    # anything is allocated for them
    huge = bytearray(path.read_bytes())
    huge[16:24] = (2 ** 31 - 1).to_bytes(8, "little")
    hp = tmp_path / "huge.tsim"
    hp.write_bytes(bytes(huge))
    with pytest.raises(tsim.api._lib.TsimError, match="size does not match"):
        tsim.Database(cuda_ctx, path=hp)
    db2.close()
    db.close()
