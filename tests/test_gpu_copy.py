"""th_copy: the copy kernel between device memory and pinned host memory."""

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def C():
    import torchhull_gb300 as th

    return th._C


@pytest.mark.parametrize("nbytes", [1, 15, 16, 17, 4096 + 3, (1 << 20) + 7, 64 << 20])
def test_round_trip(C, nbytes):
    g = torch.Generator().manual_seed(nbytes)
    src = torch.randint(0, 256, (nbytes,), dtype=torch.uint8, generator=g).pin_memory()
    dev = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    back = torch.zeros(nbytes, dtype=torch.uint8).pin_memory()
    C.copy_on_sms(dev, src)
    C.copy_on_sms(back, dev)
    torch.cuda.synchronize()
    assert torch.equal(dev.cpu(), src)
    assert torch.equal(back, src)


def test_unaligned_offsets(C):
    # views starting 3 and 5 bytes into their buffers take the byte path
    src = torch.arange(1000, dtype=torch.int32).view(torch.uint8).pin_memory()
    dev = torch.zeros(4010, dtype=torch.uint8, device="cuda")
    C.copy_on_sms(dev[5:5 + 3997], src[3:4000])
    torch.cuda.synchronize()
    assert torch.equal(dev[5:5 + 3997].cpu(), src[3:4000])
    assert int(dev[:5].sum()) == 0 and int(dev[5 + 3997:].sum()) == 0


def test_device_to_device_float(C):
    a = torch.randn(3, 1025, device="cuda")
    b = torch.empty_like(a)
    C.copy_on_sms(b, a)
    torch.cuda.synchronize()
    assert torch.equal(a, b)


def test_rejects(C):
    dev = torch.empty(64, dtype=torch.uint8, device="cuda")
    with pytest.raises(RuntimeError, match="pinned"):
        C.copy_on_sms(dev, torch.zeros(64, dtype=torch.uint8))
    with pytest.raises(RuntimeError, match="sizes differ"):
        C.copy_on_sms(dev, torch.zeros(63, dtype=torch.uint8).pin_memory())
    if torch.cuda.device_count() > 1:
        with pytest.raises(RuntimeError, match="one device"):
            C.copy_on_sms(dev, torch.empty(64, dtype=torch.uint8, device="cuda:1"))
    with pytest.raises(RuntimeError, match="CUDA"):
        C.copy_on_sms(torch.zeros(64, dtype=torch.uint8).pin_memory(), torch.zeros(64, dtype=torch.uint8).pin_memory())
