"""bielec_ao output streamed from the device (ss_write_bielec_ao) equals, byte for byte, the
Fortran-format writer applied to the merged ERIs and MC errors the same job returns."""
import pytest

from slater_stoch_gb300 import api, basis, configs, output

pytestmark = pytest.mark.gpu


def test_write_bielec_ao_from_device(tmp_path):
    b = configs.h2o_minimal(ng0=4)
    q = basis.build_mapping(b.n)
    with api.Context(0) as ctx:
        ctx.set_basis(b)
        ctx.set_quartets(*q)
        eri, sig = ctx.two_e_job(1.8, 5, 8192, 4, "shared", "split_bf16")
        ctx.write_bielec_ao(tmp_path / "dev.txt")
    output.write_bielec_ao(tmp_path / "ref.txt", q, eri, sig)
    assert (tmp_path / "dev.txt").read_bytes() == (tmp_path / "ref.txt").read_bytes()
