"""Atomic elements for the DCS path.

`STANDARD_ROCK` and `MUON_MASS` are the reference's constants
(src/noa/pms/physics.hh:58, 67-71).  The reference defines no other element;
the batched multi-element workload needs ten, so the table below takes A from
the IUPAC standard atomic weights and I (mean excitation energy) from the PDG
"Atomic and nuclear properties of materials" tables, converted to GeV.  The
Z = 11 entry is standard rock itself (A = 22, I = 136.4 eV), as in the
reference, not sodium.
"""
from dataclasses import dataclass

ELECTRON_MASS = 0.510998910E-03  # GeV, physics.hh:57
MUON_MASS = 0.10565839           # GeV, physics.hh:58
TAU_MASS = 1.77682               # GeV, physics.hh:59
X_FRACTION = 5E-02               # physics.hh:76


@dataclass(frozen=True)
class AtomicElement:
    """Mirrors noa::pms::AtomicElement {A g/mol, I GeV, Z} (physics.hh:39-43)."""
    A: float
    I: float
    Z: int


STANDARD_ROCK = AtomicElement(22.0, 0.1364E-6, 11)

# Z -> element.  A: IUPAC standard atomic weights; I: PDG mean excitation energies.
ELEMENTS = {
    1: AtomicElement(1.008, 19.2E-9, 1),       # hydrogen (H2 gas, I = 19.2 eV)
    6: AtomicElement(12.011, 78.0E-9, 6),      # carbon (graphite, I = 78.0 eV)
    8: AtomicElement(15.999, 95.0E-9, 8),      # oxygen (O2 gas, I = 95.0 eV)
    11: STANDARD_ROCK,                         # standard rock
    13: AtomicElement(26.982, 166.0E-9, 13),   # aluminium
    14: AtomicElement(28.085, 173.0E-9, 14),   # silicon
    20: AtomicElement(40.078, 191.0E-9, 20),   # calcium
    26: AtomicElement(55.845, 286.0E-9, 26),   # iron
    29: AtomicElement(63.546, 322.0E-9, 29),   # copper
    82: AtomicElement(207.2, 823.0E-9, 82),    # lead
}
BATCH_Z = (1, 6, 8, 11, 13, 14, 20, 26, 29, 82)
