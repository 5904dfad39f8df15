"""Rigid-transform helpers on the host (double precision).

exp_se3 restates xreg::ExpSE3 (lib/transforms/xregRigidUtils.cpp:40-85) and
SE3OptVarsLieAlg::operator() (lib/regi/xregSE3OptVars.cpp:128-137): a 6-vector
[w_x, w_y, w_z, v_x, v_y, v_z] -> 4x4 rigid transform.
"""
from __future__ import annotations

import numpy as np


def skew(w) -> np.ndarray:
    w = np.asarray(w, dtype=np.float64)
    return np.array([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]])


def exp_so3(W: np.ndarray) -> np.ndarray:
    """Rodrigues' formula for a skew-symmetric 3x3 W."""
    w = np.array([W[2, 1], W[0, 2], W[1, 0]])
    theta = float(np.linalg.norm(w))
    if theta < 1.0e-14:
        return np.eye(3)
    return np.eye(3) + (np.sin(theta) / theta) * W + ((1.0 - np.cos(theta)) / theta ** 2) * (W @ W)


def exp_se3(x) -> np.ndarray:
    """xreg::ExpSE3 of the Lie-algebra vector x = [w, v]."""
    x = np.asarray(x, dtype=np.float64)
    W = skew(x[:3])
    v = x[3:6]
    T = np.eye(4)
    theta = float(np.linalg.norm(x[:3]))
    if theta > 1.0e-14:
        T[:3, :3] = exp_so3(W)
        A = np.eye(3) + ((1.0 - np.cos(theta)) / theta ** 2) * W + ((theta - np.sin(theta)) / theta ** 3) * (W @ W)
        T[:3, 3] = A @ v
    else:
        T[:3, 3] = v
    return T


def euler_xyz(rx: float, ry: float, rz: float) -> np.ndarray:
    """Rotation Rz @ Ry @ Rx (radians)."""
    cx, sx, cy, sy, cz, sz = np.cos(rx), np.sin(rx), np.cos(ry), np.sin(ry), np.cos(rz), np.sin(rz)
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    return Rz @ Ry @ Rx


def rigid(R: np.ndarray, t) -> np.ndarray:
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = np.asarray(t, dtype=np.float64)
    return T


def rigid_inv(T: np.ndarray) -> np.ndarray:
    Ti = np.eye(4)
    Ti[:3, :3] = T[:3, :3].T
    Ti[:3, 3] = -T[:3, :3].T @ T[:3, 3]
    return Ti


def rot_angle_deg(R: np.ndarray) -> float:
    c = (np.trace(R) - 1.0) * 0.5
    return float(np.degrees(np.arccos(np.clip(c, -1.0, 1.0))))


def exp_se3_batch(xs) -> np.ndarray:
    """exp_se3 of every row of xs ([n, 6]) at once -> [n, 4, 4]."""
    xs = np.asarray(xs, dtype=np.float64).reshape(-1, 6)
    n = xs.shape[0]
    w, v = xs[:, :3], xs[:, 3:]
    th = np.linalg.norm(w, axis=1)
    W = np.zeros((n, 3, 3))
    W[:, 0, 1], W[:, 0, 2] = -w[:, 2], w[:, 1]
    W[:, 1, 0], W[:, 1, 2] = w[:, 2], -w[:, 0]
    W[:, 2, 0], W[:, 2, 1] = -w[:, 1], w[:, 0]
    WW = W @ W
    big = th > 1.0e-14
    ths = np.where(big, th, 1.0)
    a = np.where(big, np.sin(ths) / ths, 1.0)
    b = np.where(big, (1.0 - np.cos(ths)) / ths ** 2, 0.0)
    c = np.where(big, (ths - np.sin(ths)) / ths ** 3, 0.0)
    I = np.eye(3)[None]
    R = np.where(big[:, None, None], I + a[:, None, None] * W + b[:, None, None] * WW, I)
    A = np.where(big[:, None, None], I + b[:, None, None] * W + c[:, None, None] * WW, I)
    T = np.zeros((n, 4, 4))
    T[:, :3, :3] = R
    T[:, :3, 3] = np.einsum("nij,nj->ni", A, v)
    T[:, 3, 3] = 1.0
    return T
