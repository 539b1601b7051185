"""CPU restatement of the two PRK kernels next to the stencil (test infrastructure only).

nstream    Cxx11/nstream-cuda.cu:68-76: A[i] += B[i] + scalar * C[i], each product and sum rounded
           on its own (numpy evaluates scalar * C, then B + that, then A + that, in float64).
           Validation as :188-209: A = 0, B = C = 2, scalar = 3, checksum of |A| against
           ar = length * sum over iterations+1 of (2 + 3 * 2), relative error <= 1e-8.
transpose  Cxx11/transpose-cuda.cu:63-86 (accumulate form): B += A^T, then A += 1. Validation as
           :207-212 and :262-282: A[j][i] = order * j + i, B = 0; after iterations+1 applications
           B[j][i] must equal (i * order + j) * (iterations + 1) + (iterations + 1) * iterations / 2,
           the sum of absolute differences below 1e-8.

Only the tests use this module.
"""
from __future__ import annotations

import numpy as np


def nstream(A: np.ndarray, B: np.ndarray, C: np.ndarray, scalar: float) -> None:
    A += B + scalar * C


def nstream_checksum(length: int, iterations: int, scalar: float = 3.0, b: float = 2.0, c: float = 2.0) -> float:
    ar = 0.0
    for _ in range(iterations + 1):
        ar += b + scalar * c
    return ar * length


def nstream_validates(A: np.ndarray, iterations: int, scalar: float = 3.0) -> bool:
    ar = nstream_checksum(A.size, iterations, scalar)
    asum = float(np.abs(A).sum())
    return abs(ar - asum) / asum <= 1e-8


def transpose(A: np.ndarray, B: np.ndarray) -> None:
    B += A.T
    A += 1.0


def transpose_init(order: int) -> tuple[np.ndarray, np.ndarray]:
    j, i = np.meshgrid(np.arange(order), np.arange(order), indexing="ij")
    return (order * j + i).astype(np.float64), np.zeros((order, order))


def transpose_abserr(B: np.ndarray, iterations: int) -> float:
    order = B.shape[0]
    addit = (iterations + 1.0) * (iterations / 2.0)
    j, i = np.meshgrid(np.arange(order), np.arange(order), indexing="ij")
    reference = (i * order + j).astype(np.float64) * (1.0 + iterations) + addit
    return float(np.abs(B - reference).sum())
