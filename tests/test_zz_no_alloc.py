"""moc_fission_source_total_noalloc: the entry point for callers that own
their device arrays but cannot allocate device memory (their GPU memory is
held by another framework's pool allocator, or they sit on a latency-critical
path that cannot take cudaMalloc's implicit synchronisation).  It uses a
fixed scratch array inside the library instead of allocating.

Checked through the C ABI against the existing entry point that computes the
same quantity from the solver's own device arrays
(moc_compute_fsr_fission_rates, summed), on two calls in a row, with flux
rows packed (ld = num_groups) and padded (ld > num_groups, as the solver's
own rows are); for the clear error on sizes beyond its scratch, on host
memory, and for the NaN an out-of-range material id gives.  This file is collected last so a
run that stops at the first failure has run every other test already."""
import ctypes
import math

import numpy as np
import pytest

from conftest import load_case
from openmoc_gb300 import GB300Solver, _native, lattice

pytestmark = pytest.mark.gpu

MAX_FSRS = 1 << 19


def _expected(problem, flux):
    s = GB300Solver(problem)
    s.setFluxes(flux)
    rates = s.computeFSRFissionRates(problem.num_fsrs, nu=True)
    s.close()
    return math.fsum(rates.tolist())


def _device_args(torch, p, flux, ld=None):
    G = p.num_groups
    ld = ld or G
    rows = np.zeros((p.num_fsrs, ld), np.float32)
    rows[:, :G] = np.asarray(flux, np.float32).reshape(p.num_fsrs, G)
    # the padding holds values that must not be read
    rows[:, G:] = 1e30
    phi = torch.tensor(rows, device="cuda")
    nf = torch.tensor(p.nu_sigma_f.reshape(p.num_materials, G), device="cuda")
    mat = torch.tensor(p.fsr_mat, device="cuda")
    vol = torch.tensor(p.fsr_vol, device="cuda")
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    return phi, nf, mat, vol, out


def _call(lib, p, phi, ld, nf, mat, vol, out, stream=None, num_fsrs=None,
          num_materials=None):
    return lib.moc_fission_source_total_noalloc(
        phi.data_ptr(), ld, nf.data_ptr(),
        p.num_materials if num_materials is None else num_materials,
        mat.data_ptr(), vol.data_ptr(),
        p.num_fsrs if num_fsrs is None else num_fsrs, p.num_groups,
        None if stream is None else ctypes.c_void_p(stream),
        out if isinstance(out, int) else out.data_ptr())


@pytest.mark.parametrize("padded", [False, True])
@pytest.mark.parametrize("case", ["lat3_g2_vac", "assembly_17x17"])
def test_noalloc_total_matches_existing_entry_point_twice(case, padded):
    torch = pytest.importorskip("torch")
    if case == "assembly_17x17":
        p = lattice.assembly_17x17()
        rng = np.random.default_rng(3)
        flux = rng.uniform(0.1, 2.0, p.num_fsrs * p.num_groups).astype(np.float32)
    else:
        p, _, arr = load_case(case, "f32")
        flux = arr["probe_phi_in"]
    expected = _expected(p, flux)
    lib = _native.lib()
    ld = p.num_groups + (3 if padded else 0)
    phi, nf, mat, vol, out = _device_args(torch, p, flux, ld)
    stream = torch.cuda.current_stream().cuda_stream
    results = []
    for _ in range(2):
        out.fill_(-1.0)
        st = _call(lib, p, phi, ld, nf, mat, vol, out, stream)
        assert st == 0, lib.moc_last_error().decode()
        torch.cuda.synchronize()
        results.append(out.item())
    for got in results:
        assert got == pytest.approx(expected, rel=1e-12)
    assert results[0] == results[1]   # deterministic sum


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    p, _, arr = load_case("pin_c5g7", "f32")
    lib = _native.lib()
    G = p.num_groups
    phi, nf, mat, vol, out = _device_args(torch, p, arr["probe_phi_in"])
    st = _call(lib, p, phi, G, nf, mat, vol, out, num_fsrs=MAX_FSRS + 1)
    assert st == -1
    assert "524288" in lib.moc_last_error().decode()
    # host memory is refused, not dereferenced
    host = np.zeros(4, np.float64)
    st = _call(lib, p, phi, G, nf, mat, vol, host.ctypes.data)
    assert st == -1
    assert "device memory" in lib.moc_last_error().decode()


def test_noalloc_out_of_range_material_gives_nan():
    """A material id at or beyond num_materials is not read through: the
    FSR's rate and so the total become NaN."""
    torch = pytest.importorskip("torch")
    p, _, arr = load_case("pin_c5g7", "f32")
    lib = _native.lib()
    G = p.num_groups
    phi, nf, mat, vol, out = _device_args(torch, p, arr["probe_phi_in"])
    first = int(p.fsr_mat[0])
    mat[0] = p.num_materials
    st = _call(lib, p, phi, G, nf, mat, vol, out)
    assert st == 0, lib.moc_last_error().decode()
    torch.cuda.synchronize()
    assert math.isnan(out.item())
    # the next call with the valid ids gives the sum again
    mat[0] = first
    st = _call(lib, p, phi, G, nf, mat, vol, out)
    assert st == 0
    torch.cuda.synchronize()
    assert out.item() == pytest.approx(_expected(p, arr["probe_phi_in"]), rel=1e-12)
