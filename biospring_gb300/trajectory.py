"""Trajectory and energy output from the frame recorder (bs_set_frames / bs_read_frames).

The device writes frames into a host ring while it steps; :class:`FrameWriter` drains the ring on a
background thread and appends each frame to a PDB trajectory (one MODEL per frame), to an XTC
trajectory (bs_xtc_encode_frame, with the reference's conventions: src/IO/modern/
XTCTrajectoryWriter.cpp:15-32) and its energies to a tab-separated table laid out like the
reference's CSV sampling (step, frame rate, then one column per enabled energy term;
src/IO/CSVSampleWriter.cpp), so the stepping loop never waits for file output.
"""

from __future__ import annotations

import threading
import time

import numpy as np

from . import capi

ENERGY_LABELS = {
    "kinetic": "Kinetic energy (kJ.mol-1)",
    "spring": "Spring energy (kJ.mol-1)",
    "steric": "Steric energy (kJ.mol-1)",
    "electrostatic": "Electrostatic energy (kJ.mol-1)",
    "imp": "IMP energy (kJ.mol-1)",
    "hydrophobic": "Hydrophobic energy (kJ.mol-1)",
}


def pdb_model(model: int, xyz: np.ndarray, names=None, resnames=None, resids=None, chains=None) -> str:
    """One MODEL of ATOM records (fixed PDB columns: serial 7-11, name 13-16, residue name 18-20,
    chain 22, residue number 23-26, x y z 31-54 with 3 decimals), ENDMDL."""
    n = xyz.shape[0]
    names = names if names is not None else ["CA"] * n
    resnames = resnames if resnames is not None else ["UNK"] * n
    resids = resids if resids is not None else np.arange(1, n + 1)
    chains = chains if chains is not None else ["A"] * n
    lines = [f"MODEL    {model:5d}"]
    for i in range(n):
        nm = str(names[i])
        nm = f" {nm:<3.3s}" if len(nm) < 4 else f"{nm:<4.4s}"
        x, y, z = (float(v) for v in xyz[i])
        lines.append(f"ATOM  {(i + 1) % 100000:5d} {nm} {str(resnames[i]):>3.3s} {str(chains[i])[:1]:1s}"
                     f"{int(resids[i]) % 10000:4d}    {x:8.3f}{y:8.3f}{z:8.3f}  1.00  0.00")
    lines.append("ENDMDL")
    return "\n".join(lines) + "\n"


def xtc_frame(frame: int, xyz_angstrom: np.ndarray) -> bytes:
    """One XTC frame as the reference's XTC writer makes it: coordinates divided by 10 in double
    and stored as float (nm), an identity box, the writer's frame counter (from 0) as step and
    time, precision 1000."""
    nm = (np.asarray(xyz_angstrom, np.float32).astype(np.float64) / 10.0).astype(np.float32)
    return capi.xtc_encode(nm, int(frame), float(frame), np.eye(3, dtype=np.float32), 1000.0)


def energy_header(terms) -> str:
    return "\t".join(["# Step", "FrameRate(Hz)"] + [ENERGY_LABELS[t] for t in terms]) + "\n"


def energy_row(step: int, rate: float, energies, terms) -> str:
    idx = [capi.ENERGY_NAMES.index(t) for t in terms]
    return "\t".join([str(int(step)), f"{rate:g}"] + [repr(float(energies[k])) for k in idx]) + "\n"


def enabled_terms(config: dict) -> list:
    """The energy columns the reference writes for a configuration (kinetic always)."""
    terms = ["kinetic"]
    for key, term in (("spring_enable", "spring"), ("steric_enable", "steric"), ("coulomb_enable", "electrostatic"),
                      ("impala_enable", "imp"), ("hydrophobicity_enable", "hydrophobic")):
        if config.get(key):
            terms.append(term)
    return terms


class FrameWriter:
    """Drains a network's frame ring on a background thread into a PDB trajectory and/or an
    energy table. Call :meth:`close` after the last step (it takes the frames still in the ring)."""

    def __init__(self, net, pdb_path=None, energy_path=None, terms=None, poll: float = 0.002, names=None,
                 resnames=None, resids=None, chains=None, xtc_path=None):
        self.net = net
        self.terms = terms or ["kinetic", "spring", "steric", "electrostatic", "imp", "hydrophobic"]
        self.pdb = open(pdb_path, "w") if pdb_path else None
        self.xtc = open(xtc_path, "wb") if xtc_path else None
        self.csv = open(energy_path, "w") if energy_path else None
        if self.csv:
            self.csv.write(energy_header(self.terms))
        self.meta = dict(names=names, resnames=resnames, resids=resids, chains=chains)
        self.poll = poll
        self.frames = 0
        self.dropped = 0
        self._stop = threading.Event()
        self._last = time.perf_counter()
        self._thread = threading.Thread(target=self._run, daemon=True)
        self._thread.start()

    def _drain(self) -> int:
        steps, xyz, en, lost = self.net.readFrames(64)
        self.dropped += lost
        now = time.perf_counter()
        rate = len(steps) / (now - self._last) if len(steps) and now > self._last else 0.0
        if len(steps):
            self._last = now
        for k in range(len(steps)):
            self.frames += 1
            if self.pdb:
                self.pdb.write(pdb_model(self.frames, xyz[k], **self.meta))
            if self.xtc:
                self.xtc.write(xtc_frame(self.frames - 1, xyz[k]))
            if self.csv:
                self.csv.write(energy_row(steps[k], rate, en[k], self.terms))
        return len(steps)

    def _run(self):
        while not self._stop.is_set():
            if self._drain() == 0:
                time.sleep(self.poll)

    def close(self):
        self._stop.set()
        self._thread.join()
        self.net.synchronize()
        while self._drain():
            pass
        for f in (self.pdb, self.csv, self.xtc):
            if f:
                f.close()
        return self.frames, self.dropped
