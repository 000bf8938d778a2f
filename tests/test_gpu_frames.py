"""The frame recorder: positions and energies written by the device into a host ring while it
steps (bs_set_frames / bs_read_frames), against a handle stopped at every frame step."""

from __future__ import annotations

import time

import numpy as np
import pytest

from biospring_gb300 import BsError
from biospring_gb300 import workloads as W
from helpers import gpu_network

pytestmark = pytest.mark.gpu


def _system(**upd):
    s = W.ca_network(n=3000, seed=12)
    rng = np.random.default_rng(5)
    s.charge = np.where(rng.random(s.n) < 0.2, rng.choice([-1.0, 1.0], s.n), 0.0).astype(np.float32)
    s.config.update(coulomb_enable=1, coulomb_cutoff=12.0, timestep=0.05)
    s.config.update(upd)
    return s


def _stopped(s, every, nframes):
    net = gpu_network(s)
    pos, en = [], []
    for _ in range(nframes):
        net.computeStep(every)
        pos.append(net.getPositions())
        en.append(np.array(list(net.energies().values())))
    net.close()
    return np.stack(pos), np.stack(en)


def test_frames_match_stopped_run():
    s = _system()
    ref_pos, ref_en = _stopped(s, 5, 20)
    net = gpu_network(s)
    net.setFrames(5, 64)
    net.computeStep(100)
    steps, xyz, en, dropped = net.readFrames()
    assert dropped == 0
    np.testing.assert_array_equal(steps, np.arange(5, 101, 5))
    np.testing.assert_array_equal(xyz, ref_pos)
    np.testing.assert_array_equal(en, ref_en)
    assert net.readFrames()[0].size == 0  # nothing new
    net.close()


def test_ring_overrun_reports_drops():
    s = _system()
    net = gpu_network(s)
    net.setFrames(5, 4)
    net.computeStep(100)
    steps, xyz, en, dropped = net.readFrames()
    assert dropped == 16
    np.testing.assert_array_equal(steps, [85, 90, 95, 100])
    ref_pos, _ = _stopped(s, 5, 20)
    np.testing.assert_array_equal(xyz, ref_pos[-4:])
    net.close()


def test_reading_while_the_device_steps():
    """Frames are taken while queued steps run (no synchronisation), in order and complete."""
    s = _system()
    net = gpu_network(s)
    net.setFrames(10, 64)
    net.computeStepAsync(400)
    got_steps, got_xyz = [], []
    t0 = time.time()
    while len(got_steps) < 40 and time.time() - t0 < 60:
        st, xyz, _, dropped = net.readFrames()
        assert dropped == 0
        got_steps.extend(st.tolist())
        got_xyz.extend(list(xyz))
    net.synchronize()
    st, xyz, _, _ = net.readFrames()
    got_steps.extend(st.tolist())
    got_xyz.extend(list(xyz))
    assert got_steps == list(range(10, 401, 10))
    ref_pos, _ = _stopped(s, 10, 40)
    np.testing.assert_array_equal(np.stack(got_xyz), ref_pos)
    net.close()


def test_frames_across_stale_list_rebuilds():
    """A long timestep and a thin skin make lists go stale between planned rebuilds; each frame
    is still written once, at its step."""
    s = _system(timestep=0.5, list_skin=0.05)
    s.k = s.k * 50.0
    ref_pos, ref_en = _stopped(s, 3, 15)
    net = gpu_network(s)
    net.setFrames(3, 32)
    net.computeStep(45)
    steps, xyz, en, dropped = net.readFrames()
    assert dropped == 0
    np.testing.assert_array_equal(steps, np.arange(3, 46, 3))
    np.testing.assert_array_equal(xyz, ref_pos)
    np.testing.assert_array_equal(en, ref_en)
    net.close()


def test_frames_off_and_errors():
    s = _system()
    net = gpu_network(s)
    with pytest.raises(BsError):
        net.readFrames()
    with pytest.raises(BsError):
        net.setFrames(5, 0)
    net.setFrames(5, 8)
    net.computeStep(10)
    assert net.readFrames()[0].tolist() == [5, 10]
    net.setFrames(0, 0)
    net.computeStep(10)
    with pytest.raises(BsError):
        net.readFrames()
    net.close()


def test_frame_writer_files(tmp_path):
    """The background writer turns the ring into a PDB trajectory and an energy table while the
    handle steps."""
    from biospring_gb300.trajectory import FrameWriter, enabled_terms
    s = _system()
    ref_pos, ref_en = _stopped(s, 10, 12)
    net = gpu_network(s)
    net.setFrames(10, 64)
    terms = enabled_terms(s.config)
    w = FrameWriter(net, str(tmp_path / "t.pdb"), str(tmp_path / "e.csv"), terms=terms)
    for _ in range(4):
        net.computeStep(30)
    frames, dropped = w.close()
    assert (frames, dropped) == (12, 0)
    models = (tmp_path / "t.pdb").read_text().split("ENDMDL\n")[:-1]
    assert len(models) == 12
    for k, m in enumerate(models):
        atoms = [ln for ln in m.splitlines() if ln.startswith("ATOM")]
        xyz = np.array([[float(ln[30:38]), float(ln[38:46]), float(ln[46:54])] for ln in atoms])
        assert np.abs(xyz - ref_pos[k]).max() <= 5e-4 + 1e-6
    rows = [ln.split("\t") for ln in (tmp_path / "e.csv").read_text().splitlines()[1:]]
    assert [int(r[0]) for r in rows] == list(range(10, 121, 10))
    idx = [["kinetic", "spring", "steric", "electrostatic", "imp", "hydrophobic"].index(t) for t in terms]
    np.testing.assert_array_equal(np.array([[float(v) for v in r[2:]] for r in rows]), ref_en[:, idx])
    net.close()
