"""Dump writer and reader round trip (CPU)."""
import numpy as np

from apophis_gb300 import output, problems


def test_dump_round_trip(tmp_path):
    cfg, cons = problems.kh3d(n=32, block=16, ng=4)
    base = str(tmp_path / "kh")
    output.write_dump(base, cfg, cons, 0.5, 7)
    d = output.Dump(base + ".json")
    assert d.Time == 0.5 and d.NCycle == 7
    sk, sj, si = cfg.interior
    assert np.array_equal(d.Get("cons", flatten=False), cons[:, :, sk, sj, si])
    assert d.Get("cons").shape == (cfg.nblocks, 16 ** 3, 5)
    z, y, x = d.GetVolumeLocations(flatten=False)
    for b in range(cfg.nblocks):
        cx, cy, cz = cfg.cell_centers(b)
        assert np.array_equal(x[b], cx) and np.array_equal(y[b], cy) and np.array_equal(z[b], cz)
