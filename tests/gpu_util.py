"""Helpers shared by the GPU parity tests."""
import numpy as np
import torch

from bitwise_spgemm_gb300 import workloads as W


def dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def words_dev(words):
    return torch.from_numpy(np.ascontiguousarray(words).view(np.int32)).cuda()


def words_host(t):
    return t.cpu().numpy().view(np.uint32)


def bf16_dev(bits_u16):
    return torch.from_numpy(np.ascontiguousarray(bits_u16).view(np.int16)).cuda().view(torch.bfloat16)


def bf16_to_f32(bits_u16):
    return W.bf16_bits_to_f32(bits_u16)
