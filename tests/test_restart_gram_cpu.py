"""The thick restart's Gram block from the projection (krylov.cu k_eig_gram_proj), checked on the host in
numpy: for FP32 basis vectors V with Gram deviation E = V^T V - I and a restart V' = V Ys computed in FP32
(Ys = the FP64 rotation Y rounded to FP32, as the restart applies it), the block Ys^T (I + E) Ys differs from
the measured V'^T V' only by the roundings of the restart's own sums, which are independent from element to
element: far below the FP32 orthogonality level that E itself carries."""
import numpy as np


def test_projected_gram_block_matches_measured_fp32():
    rng = np.random.default_rng(5)
    n, nb, k = 200_000, 19, 12
    # an FP32 basis orthonormal to about its own rounding (QR in FP64, rounded)
    q, _ = np.linalg.qr(rng.standard_normal((n, nb)))
    V = q.astype(np.float32)
    V64 = V.astype(np.float64)
    E = V64.T @ V64 - np.eye(nb)
    # a rotation of the projected problem (orthonormal in FP64), rounded as the restart applies it
    y, _ = np.linalg.qr(rng.standard_normal((nb, nb)))
    Ys = y[:, :k].astype(np.float32).astype(np.float64)
    Vn = (V @ Ys.astype(np.float32)).astype(np.float64)  # the restart's FP32 sums
    measured = Vn.T @ Vn - np.eye(k)
    projected = Ys.T @ (np.eye(nb) + E) @ Ys - np.eye(k)
    dev = np.abs(measured - projected).max()
    # the block is at the level of FP32 rounding (the rounded rotation's columns are not quite orthonormal);
    # the projection captures it and misses only the restart's own roundings (~eps sqrt(nb / n)): well below
    # FP32's unit roundoff, the accuracy the one-pass orthogonalisation works to (measured here: 9e-10
    # against a block of 3e-8)
    assert np.abs(measured).max() > 1e-8
    assert dev < 0.1 * np.abs(measured).max()
    assert dev < 0.05 * np.finfo(np.float32).eps
