"""The walker state a model caches is bound to one configuration tensor: a new
tensor at a recycled address (the previous one freed) must not reuse it."""
import torch

from vmc_torch_gb300.models import WalkerState


def test_binding_follows_the_tensor_object_not_its_address():
    st = WalkerState(4, 8, torch.device("cpu"))
    a = torch.zeros((4, 8), dtype=torch.int64)
    st.bind(a)
    assert st.bound_to(a)
    a.add_(1)                        # in-place change: version moves on
    assert not st.bound_to(a)
    st.bind(a)
    ptr = a.data_ptr()
    del a
    b = torch.zeros((4, 8), dtype=torch.int64)   # typically lands at the freed address
    assert not st.bound_to(b)
    if b.data_ptr() == ptr:          # the case the weak reference exists for
        assert b._version == 0
