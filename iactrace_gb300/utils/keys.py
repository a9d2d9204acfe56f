"""Deterministic random keys, standing in for jax.random keys.

A key is a 64-bit integer; ``split`` derives independent child keys with the
SplitMix64 finaliser (Steele, Lea, Flood 2014), ``generator`` seeds a
torch.Generator from a key. Streams differ from JAX's threefry streams:
render parity is defined on the sample arrays, which are fed explicitly.
"""
from __future__ import annotations

import torch

_MASK = (1 << 64) - 1


def _mix(z: int) -> int:
    z = (z + 0x9E3779B97F4A7C15) & _MASK
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
    return z ^ (z >> 31)


class Key:
    __slots__ = ("value",)

    def __init__(self, value: int):
        self.value = int(value) & _MASK

    def __repr__(self):
        return f"Key({self.value:#x})"


def key(seed: int = 0) -> Key:
    return Key(_mix(int(seed)))


def as_key(k) -> Key:
    if k is None:
        return key(0)
    if isinstance(k, Key):
        return k
    return key(int(k))


def split(k, num: int = 2) -> list[Key]:
    k = as_key(k)
    return [Key(_mix(k.value ^ _mix(i + 1))) for i in range(num)]


def generator(k, device="cpu") -> torch.Generator:
    g = torch.Generator(device=device)
    g.manual_seed(as_key(k).value & ((1 << 63) - 1))
    return g
