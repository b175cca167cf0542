"""Device plumbing: torch tensors as owned device buffers, raw pointers, streams."""
import numpy as np
import torch


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("scatter_gb300 needs a CUDA device (GB300, sm_103a); no CPU fallback exists")


def device():
    require_cuda()
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr():
    return torch.cuda.current_stream().cuda_stream


def ptr(t):
    return None if t is None else t.data_ptr()


def to_dev(a, dtype):
    """numpy -> contiguous device tensor of ``dtype``."""
    return torch.as_tensor(np.ascontiguousarray(a)).to(device=device(), dtype=dtype).contiguous()


def empty(n, dtype):
    return torch.empty(int(n), dtype=dtype, device=device())


def zeros(n, dtype):
    return torch.zeros(int(n), dtype=dtype, device=device())


def host(t):
    return t.detach().cpu().numpy()
