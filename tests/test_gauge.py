"""U(1) gauge-field utilities (u1_utils.cpp) against the reference's outputs (golden
fixtures): the oracle bit for bit, the library's text I/O and gauge-transform generator on
the host, and the device kernels (plaquette, topological charge, gauge transform, APE
smearing) on the GPU.

Bars: oracle bit-exact; write_gauge_u1 text identical to the reference's; read_gauge_u1
within 1 ulp of the reference's read (the same text through cos / sin); rand_trans_u1 the same
phases (same std::mt19937 stream) within 1 ulp; device plaquette and topological charge within 1e-13 (absolute:
both are sums of O(V) unit-size terms in another order), gauge transform within 1e-15 per
link, APE smearing within 1e-13 per link (three sweeps of atan2, sin, cos on the device)."""
from __future__ import annotations

import os

import numpy as np
import pytest

LATS = {"l32": (32, 32), "l12x6": (12, 6), "g16": (16, 16)}


@pytest.mark.parametrize("key", list(LATS))
def test_oracle_gauge_utilities_bit_exact(oracle, golden, key):
    vec, cases = golden
    lx, ly = LATS[key]
    U, c = vec[f"{key}_links"], cases[f"{key}_gauge"]
    assert oracle.plaquette(U, lx, ly) == complex(*c["plaquette"])
    assert oracle.topo(U, lx, ly) == c["topo"]
    assert np.array_equal(oracle.gauge_trans(U, vec[f"{key}_trans"], lx, ly), vec[f"{key}_links_trans"])
    assert np.array_equal(oracle.ape_smear(U, lx, ly, 0.5, 3), vec[f"{key}_ape"])


def test_gauge_invariance_of_reference_values(oracle, golden):
    """The plaquette and the topological charge are gauge invariant (the reference's own
    transformed fields give the same values to rounding)."""
    vec, cases = golden
    for key, (lx, ly) in LATS.items():
        Ut = vec[f"{key}_links_trans"]
        assert abs(oracle.plaquette(Ut, lx, ly) - complex(*cases[f"{key}_gauge"]["plaquette"])) < 1e-14
        assert abs(oracle.topo(Ut, lx, ly) - cases[f"{key}_gauge"]["topo"]) < 1e-12


def test_write_and_read_gauge_text(gl, golden, tmp_path):
    vec, cases = golden
    path = os.path.join(tmp_path, "g16.dat")
    gl.write_gauge_u1(vec["g16_links"], 16, 16, path)
    assert open(path).read() == cases["g16_gauge"]["text"]
    U = np.zeros(2 * 256, np.complex128)
    gl.read_gauge_u1(U, 16, 16, path)
    assert np.max(np.abs(U - vec["g16_links_read"])) <= 2.3e-16


def test_read_gauge_short_file_is_an_error(gl, tmp_path):
    path = os.path.join(tmp_path, "short.dat")
    with open(path, "w") as f:
        f.write("0.1\n0.2\n")
    with pytest.raises(gl.GlinalgError):
        gl.read_gauge_u1(np.zeros(2 * 16, np.complex128), 4, 4, path)


def test_rand_trans_matches_reference(gl, golden):
    """The same phases from the same std::mt19937 stream; cos / sin of another libm (the
    fixtures were written on x86-64) may differ in the last bit."""
    vec, _ = golden
    for key, (lx, ly) in LATS.items():
        assert np.max(np.abs(gl.Generator(99).rand_trans_u1(lx, ly) - vec[f"{key}_trans"])) <= 2.3e-16


def test_unit_gauge_host(gl):
    U = np.zeros(2 * 12, np.complex128)
    gl.unit_gauge_u1(U, 4, 3)
    assert np.all(U == 1.0)


@pytest.mark.gpu
@pytest.mark.parametrize("key", list(LATS))
def test_device_gauge_utilities_match_reference(gl, gpu, golden, key):
    import torch
    vec, cases = golden
    lx, ly = LATS[key]
    U, c = vec[f"{key}_links"], cases[f"{key}_gauge"]
    assert abs(gl.get_plaquette_u1(U, lx, ly) - complex(*c["plaquette"])) < 1e-13
    assert abs(gl.get_topo_u1(U, lx, ly) - c["topo"]) < 1e-13
    Ut = U.copy()
    gl.apply_gauge_trans_u1(Ut, vec[f"{key}_trans"], lx, ly)
    assert np.max(np.abs(Ut - vec[f"{key}_links_trans"])) < 1e-15
    S = np.zeros_like(U)
    gl.apply_ape_smear_u1(S, U, lx, ly, 0.5, 3)
    assert np.max(np.abs(S - vec[f"{key}_ape"])) < 1e-13
    # the same on device-resident tensors
    Ud = torch.from_numpy(U).to(gpu)
    Sd = torch.zeros_like(Ud)
    gl.apply_ape_smear_u1(Sd, Ud, lx, ly, 0.5, 3)
    assert np.max(np.abs(Sd.cpu().numpy() - vec[f"{key}_ape"])) < 1e-13
    assert abs(gl.get_plaquette_u1(Ud, lx, ly) - complex(*c["plaquette"])) < 1e-13


@pytest.mark.gpu
def test_device_gauge_invariance_1024(gl, gpu):
    """At 1024^2: a random gauge transform leaves the plaquette and the topological charge
    unchanged, and the staggered operator is covariant: D[U^g] (g psi) = g (D[U] psi)."""
    import torch
    lx = ly = 1024
    g = gl.Generator(1337)
    U = torch.from_numpy(g.rand_gauge_u1(lx, ly)).to(gpu)
    gt = torch.from_numpy(g.rand_trans_u1(lx, ly)).to(gpu)
    p0, q0 = gl.get_plaquette_u1(U, lx, ly), gl.get_topo_u1(U, lx, ly)
    Ut = U.clone()
    gl.apply_gauge_trans_u1(Ut, gt, lx, ly)
    assert abs(gl.get_plaquette_u1(Ut, lx, ly) - p0) < 1e-12
    assert abs(gl.get_topo_u1(Ut, lx, ly) - q0) < 1e-9
    assert abs(q0 - round(q0)) < 1e-9  # an integer on a periodic lattice
    psi = torch.from_numpy(g.gaussian(lx * ly)).to(gpu)
    a, b = torch.zeros_like(psi), torch.zeros_like(psi)
    gl.Operator(0, lx, ly, 0.01, U).apply(a, psi)
    gl.Operator(0, lx, ly, 0.01, Ut).apply(b, gt * psi)
    assert (torch.linalg.vector_norm(b - gt * a) / torch.linalg.vector_norm(a)).item() < 1e-14
    one = torch.zeros_like(U)
    gl.unit_gauge_u1(one, lx, ly)
    assert abs(gl.get_plaquette_u1(one, lx, ly) - 1.0) < 1e-15
