"""Benchmark-case vocabulary accepted by the GB300 hot path.

Field names and meanings follow the reference's frozen configuration
dataclasses (``src/isogrid/config/model.py:12-63``) so that a caller holding a
reference ``BenchmarkCase`` can pass it unchanged: every function in this
package reads only ``case.geometry.atoms[i].element``, ``.position``,
``case.geometry.unit``, ``case.charge``, ``case.spin_states`` and
``case.reference_model.xc``/``.pseudo`` (duck typing).
"""

from __future__ import annotations

import math
from dataclasses import dataclass

Coordinate3D = tuple[float, float, float]


@dataclass(frozen=True)
class AtomSpec:
    element: str
    position: Coordinate3D


@dataclass(frozen=True)
class MoleculeGeometry:
    name: str
    atoms: tuple[AtomSpec, ...]
    unit: str


@dataclass(frozen=True)
class SpinStateSpec:
    label: str
    spin: int


@dataclass(frozen=True)
class ReferenceModelSettings:
    mean_field: str
    basis: str
    pseudo: str
    xc: str


@dataclass(frozen=True)
class ScfSettings:
    conv_tol: float
    max_cycle: int


@dataclass(frozen=True)
class BenchmarkCase:
    name: str
    description: str
    geometry: MoleculeGeometry
    charge: int
    spin_states: tuple[SpinStateSpec, ...]
    reference_model: ReferenceModelSettings
    scf: ScfSettings


_STAGE1_MODEL = ReferenceModelSettings(mean_field="uks", basis="gth-dzvp", pseudo="gth-pade", xc="lda,vwn")
_STAGE1_SCF = ScfSettings(conv_tol=1.0e-10, max_cycle=100)
_SINGLET_TRIPLET = (SpinStateSpec("singlet", 0), SpinStateSpec("triplet", 2))


def make_h2_case(bond_length_bohr: float = 1.4, name: str | None = None) -> BenchmarkCase:
    """H2 on the z axis at +-R/2 (reference default R = 1.4 Bohr, ``config/defaults.py:46-67``)."""

    half = 0.5 * float(bond_length_bohr)
    return BenchmarkCase(
        name=name or f"h2_r{bond_length_bohr:g}_bohr",
        description="H2 dimer on the z axis.",
        geometry=MoleculeGeometry(
            name="H2",
            atoms=(AtomSpec("H", (0.0, 0.0, -half)), AtomSpec("H", (0.0, 0.0, half))),
            unit="Bohr",
        ),
        charge=0,
        spin_states=_SINGLET_TRIPLET,
        reference_model=_STAGE1_MODEL,
        scf=_STAGE1_SCF,
    )


H2_BOND_LENGTH_BOHR = 1.4
H2_BENCHMARK_CASE = make_h2_case(H2_BOND_LENGTH_BOHR, name="h2_r1p4_bohr")


def make_molecule_case(name: str, atoms: list[tuple[str, Coordinate3D]], spin: int = 0) -> BenchmarkCase:
    """Generic neutral closed- or open-shell case built from (element, position) pairs."""

    return BenchmarkCase(
        name=name.lower(),
        description=f"{name} synthetic case.",
        geometry=MoleculeGeometry(
            name=name,
            atoms=tuple(AtomSpec(el, tuple(float(c) for c in pos)) for el, pos in atoms),
            unit="Bohr",
        ),
        charge=0,
        spin_states=(SpinStateSpec("singlet" if spin == 0 else f"spin{spin}", spin),),
        reference_model=_STAGE1_MODEL,
        scf=_STAGE1_SCF,
    )


def make_benzene_case(cc_bohr: float = 2.64, ch_bohr: float = 2.05) -> BenchmarkCase:
    """Planar hexagonal C6H6 ring in the z = 0 plane (C-C and C-H bond lengths in Bohr)."""

    atoms = []
    for i in range(6):
        phi = math.pi / 3.0 * i
        atoms.append(("C", (cc_bohr * math.cos(phi), cc_bohr * math.sin(phi), 0.0)))
    for i in range(6):
        phi = math.pi / 3.0 * i
        r = cc_bohr + ch_bohr
        atoms.append(("H", (r * math.cos(phi), r * math.sin(phi), 0.0)))
    return make_molecule_case("C6H6", atoms)


def make_h2o_case(oh_bohr: float = 1.81, angle_deg: float = 104.5) -> BenchmarkCase:
    half = 0.5 * math.radians(angle_deg)
    hx = oh_bohr * math.sin(half)
    hz = oh_bohr * math.cos(half)
    return make_molecule_case("H2O", [("O", (0.0, 0.0, 0.0)), ("H", (-hx, 0.0, hz)), ("H", (hx, 0.0, hz))])


def make_ch4_case(ch_bohr: float = 2.06) -> BenchmarkCase:
    s = ch_bohr / math.sqrt(3.0)
    return make_molecule_case(
        "CH4",
        [("C", (0.0, 0.0, 0.0)), ("H", (s, s, s)), ("H", (s, -s, -s)), ("H", (-s, s, -s)), ("H", (-s, -s, s))],
    )
