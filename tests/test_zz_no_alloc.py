"""mappg_sys_force_noalloc through the C ABI: forces, energy and virial
written into caller-owned device buffers, with every intermediate array in
the library's fixed scratch, against mappg_sys_force + mappg_sys_get_f on the
same systems.  Collected last so that it also runs after every other GPU test
in one process; it passes alone as well."""
import ctypes as C

import numpy as np
import pytest

from mapp4py_gb300 import _lib, synth

pytestmark = pytest.mark.gpu

SCRATCH_ATOMS = 1 << 18
ERR_ARG = -1  # MAPPG_ERR_ARG


def _noalloc(s):
    """One call with outputs in torch-owned device buffers pre-filled with NaN."""
    torch = pytest.importorskip("torch")
    f = torch.full((s.n, 3), float("nan"), dtype=torch.float64, device="cuda")
    ev = torch.full((7,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = _lib.load().mappg_sys_force_noalloc(s.h, C.c_void_p(f.data_ptr()), C.c_void_p(ev.data_ptr()))
    _lib.check(rc)
    s.sync()
    return f.cpu().numpy(), ev.cpu().numpy()


def _check_against_force(s):
    pe, vir = s.force()
    f = s.get_f()
    fn, ev = _noalloc(s)
    assert abs(ev[0] - pe) <= 1e-12 * abs(pe)
    assert np.max(np.abs(ev[1:] - vir)) <= 1e-11 * np.max(np.abs(vir))
    assert np.max(np.abs(fn - f)) <= 1e-10 * max(1.0, np.max(np.abs(f)))


def test_noalloc_matches_force_on_consecutive_calls(potentials):
    ff2 = _lib.ForceField.setfl(potentials[("A", "B")][0])
    ff1 = _lib.ForceField.setfl(potentials[("A",)][0])
    big = synth.alloy((5, 5, 5), xB=0.5, sigma=0.08, seed=11)
    a = _lib.System(ff2, big.H, big.x, big.elem, big.masses)
    a.build()
    _check_against_force(a)
    # a smaller system next: what the first call left in the scratch beyond
    # this system's atoms must not reach its results
    H, x = synth.fcc((4, 4, 4))
    x = x + np.random.default_rng(5).normal(0.0, 0.05, x.shape)
    b = _lib.System(ff1, H, x, np.zeros(len(x), np.uint8), [synth.MASS])
    b.build()
    _check_against_force(b)
    # and the first system again, after its atoms moved
    a.set_x(big.x + np.random.default_rng(6).normal(0.0, 0.02, big.x.shape))
    a.update()
    _check_against_force(a)


def test_noalloc_calls_after_the_first_allocate_nothing(potentials):
    """The promise itself: once the first call on the device has done its
    set-up, further calls leave the device's free memory and torch's pool
    exactly as they were."""
    torch = pytest.importorskip("torch")
    L = _lib.load()
    ff = _lib.ForceField.setfl(potentials[("A", "B")][0])
    c = synth.alloy((6, 6, 6), xB=0.4, sigma=0.06, seed=21)
    s = _lib.System(ff, c.H, c.x, c.elem, c.masses)
    s.build()
    f = torch.empty((s.n, 3), dtype=torch.float64, device="cuda")
    ev = torch.empty(7, dtype=torch.float64, device="cuda")
    fp, evp = C.c_void_p(f.data_ptr()), C.c_void_p(ev.data_ptr())
    _lib.check(L.mappg_sys_force_noalloc(s.h, fp, evp))  # first call: set-up
    s.sync()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    reserved0 = torch.cuda.memory_reserved()
    for _ in range(5):
        _lib.check(L.mappg_sys_force_noalloc(s.h, fp, evp))
    s.sync()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, "device free memory changed by %d bytes" % (free0 - free1)
    assert torch.cuda.memory_reserved() == reserved0
    pe, _ = s.force()
    assert abs(float(ev[0].item()) - pe) <= 1e-12 * abs(pe)


def test_noalloc_refuses_what_it_cannot_do(potentials):
    torch = pytest.importorskip("torch")
    L = _lib.load()
    ff = _lib.ForceField.setfl(potentials[("A",)][0])
    out = torch.empty(3 * (SCRATCH_ATOMS + 1) + 7, dtype=torch.float64, device="cuda")
    fp = C.c_void_p(out.data_ptr())
    H, x = synth.fcc((3, 3, 3))
    elem = np.zeros(len(x), np.uint8)
    s = _lib.System(ff, H, x, elem, [synth.MASS])
    assert L.mappg_sys_force_noalloc(s.h, fp, None) == ERR_ARG  # no neighbour list yet
    assert b"neighbour list" in L.mappg_last_error()
    m = _lib.System(ff, H, x, elem, [synth.MASS], precision=_lib.MIXED)
    m.build()
    assert L.mappg_sys_force_noalloc(m.h, fp, None) == ERR_ARG
    assert b"FP64" in L.mappg_last_error()
    cells = int(np.ceil((SCRATCH_ATOMS / 4) ** (1 / 3)))  # 4 atoms per FCC cell
    H, x = synth.fcc((cells,) * 3)
    assert len(x) > SCRATCH_ATOMS
    big = _lib.System(ff, H, x, np.zeros(len(x), np.uint8), [synth.MASS])
    assert L.mappg_sys_force_noalloc(big.h, fp, None) == ERR_ARG
    assert str(SCRATCH_ATOMS).encode() in L.mappg_last_error()
    assert L.mappg_sys_force_noalloc(s.h, None, None) == ERR_ARG
