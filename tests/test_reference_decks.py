"""The reference's own example decks, where its checkout is present (CPU only).

Every 3-D explicit deck under examples/input loads (mesh, material, BCs,
rigid bodies, thermal keys); the 2-D / axisymmetric ones and the legacy
Cylinder block are rejected as unsupported. The thermal two-body contact deck
Contact_Compression_tetra.json (tetra_cyl.k, Hollomon, two Plane bodies, heat
conduction) runs 1500 steps on the oracle and on the reference's own code
(the harness built from its sources) with identical results, bit for bit:
displacements, reaction history, temperatures and plastic strain.
"""
import os

import numpy as np
import pytest

import weldformfem_gb300 as wf
from oracle import orabind as O
from oracle import refbind as R
from tests import helpers as H

INPUT = os.path.join(H.REFERENCE_ROOT, "examples", "input")
pytestmark = pytest.mark.skipif(not os.path.isdir(INPUT), reason="reference examples not present")

LOADS = {  # deck: (nodes, elements, nodes per element, rigid bodies, thermal)
    "Compression_hexa.json": (6479, 5760, 8, 0, 0),
    "Compression_hexa_hollomon.json": (6479, 5760, 8, 0, 0),
    "Compression_tetra.json": (2513, 12197, 4, 0, 0),
    "Contact_Compression_tetra.json": (2513, 12197, 4, 2, 1),
    "Contact_Compression_tetra_Hollomon_rmsh.json": (2513, 12197, 4, 2, 0),
    "test_1el/test_1_elem.json": (4, 1, 4, 2, 0),
    "test_1el/test_2_elem.json": (5, 2, 4, 2, 0),
}
UNSUPPORTED = ["Compression.json", "Compression_axisymm_quad.json",
               "Contact_Compression_axisymm_quad.json", "Traction_pe.json"]


@pytest.fixture
def in_input_dir():
    # the reference driver opens mesh files relative to its working directory
    cwd = os.getcwd()
    os.chdir(INPUT)
    yield
    os.chdir(cwd)


def test_reference_decks_load(in_input_dir):
    for name, (nn, ne, npe, bodies, thermal) in LOADS.items():
        i = wf.Deck(name).info
        assert (i["nn"], i["ne"], i["npe"], i["rigid_bodies"], i["thermal"]) == \
            (nn, ne, npe, bodies, thermal), name
    for name in UNSUPPORTED:
        with pytest.raises(wf.WfError) as e:
            wf.Deck(name)
        assert e.value.status == wf.WF_ERR_UNSUPPORTED, name


@pytest.mark.skipif(not R.available(), reason="reference harness not built")
def test_thermal_contact_deck_matches_reference(in_input_dir):
    k = wf.Deck("Contact_Compression_tetra.json")
    assert k.info["thermal"] == 1 and k.info["rigid_bodies"] == 2
    res = []
    for dom in (O.OracleDomain(), R.RefDomain()):
        k.setup(dom)
        dom.init()
        dom.step(1500)
        res.append((dom.node_vec("u"), dom.reaction(), dom.node_scalar("T"),
                    dom.elem_scalar("pl_strain")))
    for a, b in zip(*res):
        np.testing.assert_array_equal(a, b)
    u, r, T, pl = res[0]
    assert pl.max() > 0 and r.max() > 0 and T.max() > T.min()
