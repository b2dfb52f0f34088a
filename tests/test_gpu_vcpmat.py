"""GPU: .vcpmat files straight to and from device memory (vcpcu_vcpmat_load_dev
/ save_dev, pinned chunks): the reference's fixture operands go to HBM, the
plain product runs there, and the file written from HBM is byte-identical to
the product file the reference wrote; a matrix of several staging chunks with
a padded leading dimension survives the round trip bit for bit."""
from pathlib import Path

import numpy as np
import pytest

from vcp_gb300 import pidcuda, vcpmat

pytestmark = pytest.mark.gpu
FIX = Path(__file__).resolve().parent / "golden" / "vcpmat"


def test_fixture_product_through_device_files(cuda_lib, tmp_path):
    import torch
    dev = torch.device("cuda")
    s = torch.cuda.current_stream()
    _, m, k = vcpmat.info(str(FIX / "A"))
    _, k2, n = vcpmat.info(str(FIX / "B"))
    A = torch.empty(2 * m * k, dtype=torch.float64, device=dev)
    B = torch.empty(2 * k * n, dtype=torch.float64, device=dev)
    C = torch.empty(2 * m * n, dtype=torch.float64, device=dev)
    vcpmat.load_dev(str(FIX / "A"), A, m, stream=s)
    vcpmat.load_dev(str(FIX / "B"), B, k, stream=s)
    pidcuda.mulmm_dev(m, n, k, A, m, B, k, C, m, pidcuda.FORM_PLAIN, 0, s)
    out = str(tmp_path / "C")
    vcpmat.save_dev(out, C, m, n, m, "interval", stream=s)
    assert Path(out + ".vcpmat").read_bytes() == (FIX / "C.vcpmat").read_bytes()


@pytest.mark.parametrize("kind", ["interval", "double", "interval_dd"])
def test_device_round_trip_multi_chunk(cuda_lib, tmp_path, kind):
    import torch
    width = {"interval": 2, "double": 1, "interval_dd": 4}[kind]
    rows, cols, ld = 1500, {"interval": 3000, "double": 6000, "interval_dd": 1500}[kind], 1531
    rng = np.random.default_rng(width)
    host = rng.standard_normal(rows * cols * width)
    name = str(tmp_path / kind)
    vcpmat.save(name, host, rows, cols, kind)
    dev = torch.device("cuda")
    s = torch.cuda.current_stream()
    D = torch.full((ld * cols * width,), float("nan"), dtype=torch.float64, device=dev)
    vcpmat.load_dev(name, D, ld, stream=s)
    got = D.view(cols, ld, width)[:, :rows, :].cpu().numpy().reshape(-1)
    assert got.tobytes() == host.tobytes()
    out = str(tmp_path / (kind + "_out"))
    vcpmat.save_dev(out, D, rows, cols, ld, kind, stream=s)
    assert Path(out + ".vcpmat").read_bytes() == Path(name + ".vcpmat").read_bytes()
