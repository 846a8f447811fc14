"""The host-side mirror of the reference's Python interface (CPU parts).

Model/ShotReceiver behave as readmodel.py:1-136; read_model (broken in the
reference, readmodel.py:70) returns the (nx, ny, nz) array.
"""
import numpy as np

import readmodel as R


def test_write_and_read_model_roundtrip(tmp_path):
    m = R.Model(nx=5, ny=4, nz=3, dx=10, dy=10, dz=10, vel_file=str(tmp_path / "v.bin"),
                rho_file=str(tmp_path / "r.bin"), epsilon_file=str(tmp_path / "e.bin"))
    m.generate_model(vel=2500, rho=1000, epsilon=0.2)
    assert (tmp_path / "v.bin").stat().st_size == 5 * 4 * 3 * 4
    assert not (tmp_path / "d.bin").exists()  # delta == 0 writes nothing (readmodel.py:54-55)
    assert np.all(m.read_model(m.vel_file) == 2500)
    a = np.arange(60, dtype=np.float32)  # file order z fastest, then x, then y
    a.tofile(tmp_path / "x.bin")
    r = m.read_model(str(tmp_path / "x.bin"))
    assert r.shape == (5, 4, 3)
    assert r[1, 2, 0] == a[0 + 3 * (1 + 5 * 2)]


def test_shot_list_and_node_split():
    sg = R.ShotReceiver(sxbeg=10, sybeg=20, szbeg=2, jsx=5, jsy=10, jsz=1, sxend=20, syend=30, szend=2,
                        dgx=10.0, dgy=10.0, dgt=0.002, shotfolder="./s/")
    assert sg.nshot == 6
    assert sg.shotlist[0] == (10, 20, 2, 5, 10, 1) and sg.shotlist[1] == (10, 30, 2, 5, 10, 1)
    tasks = sg.allocateNode(nnode=4)
    assert [len(t) for t in tasks] == [2, 2, 1, 1]
    assert tasks[1][0] == sg.shotlist[1]


def test_record_size_for_resume():
    m = R.Model(nx=21, ny=10, nz=8, dx=10, dy=10, dz=10)
    sg = R.ShotReceiver(1, 1, 1, 1, 1, 1, 1, 1, 1, dgx=20.0, dgy=10.0, dgt=0.002, shotfolder="./")
    fd = R.Acoustic3d1order(model=m, sg=sg, nt=101, dt=0.001, fpeak=20.0, snap_folder="./", snap_interval=10)
    assert fd.record_bytes() == 4 * 11 * 10 * 51
