"""The allocation-free mass integrals agree with the allocating entry point.

sb_mass_integrals_noalloc exists for callers that may not allocate device
memory when they need the answer (a framework that owns all device memory
through its own pool, a plug-in whose host application forbids device
allocations once it has started, a real-time loop that cannot pay for
cudaMalloc's implicit synchronisation).
It computes what sb_update_mass computes, from device arrays the caller
owns, with a fixed scratch array compiled into the library.  This test calls
it through the C ABI twice in a row (a second, larger grid on the second
call, so a stale scratch array would show) and compares each result with
sb_update_mass on the same fields, at 1e-9 relative: both sum the same FP32
fields in FP64, only the order of the sums differs.  Around each call the
device's free memory (cudaMemGetInfo) must not change: the call allocates
nothing.  It also checks that a grid larger than the scratch array is
refused with SB_ERR_INVALID.

It lives in its own file so that pytest collects it after every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [(64, "c0", 11), (256, "c1", 12)]


def _reference_masses(nT, recipe, seed):
    from soapbubble_gb300 import synth
    from soapbubble_gb300.bubble import GpuBubble, make_params
    f = synth.make_fields(recipe, nT, seed)
    with GpuBubble(make_params(nT, 0.005)) as gb:
        gb.upload_fields(f.eta, f.gamma, f.uth, f.uph, f.uair_init, f.vair_init)
        gb.step(2, 0.5, 0.005)
        st = gb.stats(mass=True)
        eta = gb.download("eta").astype(np.float32)
        gam = gb.download("gamma").astype(np.float32)
    return eta, gam, (st.mass_eta, st.mass_gamma)


def test_noalloc_mass_integrals_match_sb_update_mass(gpulib):
    from soapbubble_gb300 import cudart
    L = gpulib.lib()
    out_host = np.zeros(2)
    d_out = cudart.DeviceBuffer(16)
    try:
        for nT, recipe, seed in CASES:
            eta, gam, ref = _reference_masses(nT, recipe, seed)
            d_eta, d_gam = cudart.DeviceBuffer(eta.nbytes), cudart.DeviceBuffer(gam.nbytes)
            try:
                cudart.memcpy_htod(d_eta, eta)
                cudart.memcpy_htod(d_gam, gam)
                free0 = cudart.mem_get_info()[0]
                rc = L.sb_mass_integrals_noalloc(nT, d_eta.ptr, d_gam.ptr, d_out.ptr, None)
                assert rc == 0, L.sb_last_error().decode()
                cudart.memcpy_dtoh(out_host, d_out)  # ordered after the kernels
                assert cudart.mem_get_info()[0] == free0
                np.testing.assert_allclose(out_host, ref, rtol=1e-9, atol=0)
            finally:
                d_eta.free()
                d_gam.free()
    finally:
        d_out.free()


def test_noalloc_rejects_grids_beyond_its_scratch(gpulib):
    from soapbubble_gb300 import cudart
    L = gpulib.lib()
    buf = cudart.DeviceBuffer(64)
    try:
        rc = L.sb_mass_integrals_noalloc(2048, buf.ptr, buf.ptr, buf.ptr, None)
        assert rc == gpulib.SB_ERR_INVALID
        assert b"1024" in L.sb_last_error()
    finally:
        buf.free()
