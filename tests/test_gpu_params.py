"""findParams on the device (stntt_find_params_device) against the
reference's own values (findParams(2^k, 11), pinned in the golden vectors) and
against the host search for other sizes and lower bounds."""

import pytest

import stntt_gb300 as st

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def device_params(size, min_mod):
    out = torch.full((3,), -1, dtype=torch.int64, device="cuda")
    st.find_params_device(size, min_mod, out)
    torch.cuda.synchronize()
    root, mod, status = (int(v) for v in out.cpu())
    return root, mod, status


def test_device_params_match_reference(stntt_lib, golden):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    for lg, (root, mod) in golden["params"].items():
        assert device_params(1 << int(lg), 11) == (root, mod, 0), lg


@pytest.mark.parametrize("size,min_mod", [(1, 1), (1, 2), (3, 100), (1000, 100000), (12345, 10 ** 8),
                                          (1 << 20, 1 << 30), (6, 7), (1 << 27, 11)])
def test_device_params_match_host(stntt_lib, size, min_mod):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    assert device_params(size, min_mod) == (*st.findParams(size, min_mod), 0)


def test_device_params_beyond_32_bits(stntt_lib):
    """No prime k 2^31 + 1 >= 2^31 + 2 lies below 2^32 (3 2^31 + 1 does not fit):
    the kernel reports STNTT_EUNSUPPORTED (5) instead of searching on."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    assert device_params(1 << 31, (1 << 31) + 2) == (0, 0, 5)
    with pytest.raises(st.StnttError):
        st.find_params_device(1 << 32, 11, torch.empty(3, dtype=torch.int64, device="cuda"))
