"""Device-to-device state copies of the C ABI (amr_tree_load_state_device /
amr_tree_download_state_device): 16-byte-aligned buffers are copied by an SM
kernel, other buffers by the copy engines; both must move every byte of
every field, also while another stream moves data between host and device
(the pipelined feeding of runs)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def amr():
    import amr_gb300 as A

    A.lib()
    return A


@pytest.mark.parametrize("offset", [0, 8])
@pytest.mark.parametrize("fields,prec", [(1, "F32"), (1, "F64"), (4, "F64")])
def test_load_and_download_roundtrip(amr, offset, fields, prec):
    torch = pytest.importorskip("torch")
    dt = getattr(amr, prec)
    t = amr.Tree(2, 16, 1, 6, capacity=300, dtype=dt, fields=fields)
    t.refine_uniform(3)
    P = t.size
    flat = 18 * 18
    tdt = torch.float32 if prec == "F32" else torch.float64
    esize = 4 if prec == "F32" else 8
    n = fields * P * flat
    rng = np.random.default_rng(7)
    host = rng.standard_normal(n).astype(np.float32 if prec == "F32" else np.float64)
    # a device buffer whose data starts `offset` bytes past a 256-byte boundary
    raw = torch.empty(n * esize + 256, dtype=torch.uint8, device="cuda")
    src = raw[offset:offset + n * esize].view(tdt)
    src.copy_(torch.from_numpy(host).cuda())
    side = torch.cuda.Stream()
    noise = torch.empty(64 << 20, dtype=torch.uint8).pin_memory()
    dev_noise = torch.empty_like(noise, device="cuda")
    torch.cuda.synchronize()  # the source is filled before the tree's stream reads it
    with torch.cuda.stream(side):  # host traffic on another stream meanwhile
        dev_noise.copy_(noise, non_blocking=True)
    t.load_state_device(src.data_ptr(), P)
    got = t.download_state()
    np.testing.assert_array_equal(got.ravel(), host)
    raw2 = torch.zeros(n * esize + 256, dtype=torch.uint8, device="cuda")
    dst = raw2[offset:offset + n * esize].view(tdt)
    with torch.cuda.stream(side):
        noise.copy_(dev_noise, non_blocking=True)
    t.download_state_device(dst.data_ptr(), P)
    t.synchronize()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dst.cpu().numpy(), host)
    t.close()
