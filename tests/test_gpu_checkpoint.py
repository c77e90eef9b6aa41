"""Checkpoint / resume of the sweep: an orderly interruption after some waves
(PCG_ECANCELLED with the checkpoint written, a host-side stop, no device
fault) and a second call that resumes from the file give the golden value;
a checkpoint of another problem is ignored."""
import os

import pytest


@pytest.mark.gpu
def test_D_stop_and_resume(pcg, golden, tmp_path):
    g = golden["D_default"]["1000000000000000000"]
    x, y, z, k = 10 ** 18, g["y"], g["z"], g["k"]
    path = str(tmp_path / "d18.ckpt")
    with pytest.raises(pcg.PrimecountError) as e:
        pcg.D(x, y, z, k, checkpoint=path, stop_after_waves=2)
    assert e.value.status == 7
    assert os.path.exists(path)
    # a second stop further on, then the rest
    with pytest.raises(pcg.PrimecountError):
        pcg.D(x, y, z, k, checkpoint=path, stop_after_waves=2)
    assert pcg.D(x, y, z, k, checkpoint=path) == g["D"]
    assert not os.path.exists(path)
    st = pcg.last_stats()
    assert st["leaves"] == 1524253981   # counters carried over the interruptions


@pytest.mark.gpu
def test_checkpoint_of_another_problem_is_ignored(pcg, golden, tmp_path):
    g18 = golden["D_default"]["1000000000000000000"]
    g17 = golden["D_default"]["100000000000000000"]
    path = str(tmp_path / "x.ckpt")
    with pytest.raises(pcg.PrimecountError):
        pcg.D(10 ** 18, g18["y"], g18["z"], g18["k"], checkpoint=path, stop_after_waves=1)
    assert pcg.D(10 ** 17, g17["y"], g17["z"], g17["k"], checkpoint=path) == g17["D"]


@pytest.mark.gpu
def test_S2_hard_resume(pcg, golden, tmp_path):
    g = golden["S2_hard_default"]["1000000000000000000"]
    path = str(tmp_path / "s2.ckpt")
    with pytest.raises(pcg.PrimecountError):
        pcg.S2_hard(10 ** 18, g["y"], g["z"], g["c"], checkpoint=path, stop_after_waves=1)
    assert pcg.S2_hard(10 ** 18, g["y"], g["z"], g["c"], checkpoint=path) == g["S2_hard"]
