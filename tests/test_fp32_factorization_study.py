"""Why the mixed form keeps the block factorisation in FP64.

Takes real Gauss-Newton systems of the oracle (contact scene, first substep)
and solves every strand's block-tridiagonal system with the block Thomas
recurrence the solver uses, including its relative diagonal shift
max(1e-12 max|b_ii|, 1e-24) on every Schur complement B_n
(cuda_backend.cu:855-864).  The shifts of the FP64 factorisation define the
system A (the Gauss-Newton blocks plus those shifts) that every variant is
measured against:

* FP64 block Thomas;
* FP32 block Thomas (the same shifts, applied in FP32);
* FP32 block Thomas with three sweeps of FP64 iterative refinement
  (r = b - A x in FP64, x += FP32 solve of r);
* the same two with symmetric diagonal scaling (D^-1/2 A D^-1/2) before the
  FP32 factorisation.

The systems are ill-conditioned (tiny rotational inertia against stiff
stretch and shear: block condition numbers of 1e8-1e10), so an FP32
factorisation's relative residual is O(1), with or without scaling, and
FP64 refinement on top of it does not converge: an FP32 factorisation cannot
recover the FP64 direction.  Small CPU case; runs the oracle only.
"""
import ctypes

import numpy as np

import khs_native as kn
import scenes


def _shift(B):
    return max(1.0e-12 * float(np.max(np.abs(np.diag(B)))), 1.0e-24)


def _thomas(D, U, rhs, dtype, shifts=None):
    """Block Thomas solve; with ``shifts`` None the relative shift of each
    Schur complement is computed (and returned), else the given shifts are
    added."""
    n = len(D)
    D = D.astype(dtype); U = U.astype(dtype); r = rhs.astype(dtype)
    C = np.zeros_like(D); dp = np.zeros_like(r)
    used = np.zeros(n)
    for k in range(n):
        B = D[k].copy(); rr = r[k].copy()
        if k > 0:
            B -= U[k - 1].T @ C[k - 1]
            rr -= U[k - 1].T @ dp[k - 1]
        used[k] = _shift(B.astype(np.float64)) if shifts is None else shifts[k]
        B += np.eye(6, dtype=dtype) * dtype(used[k])
        inv = np.linalg.inv(B)
        if k + 1 < n:
            C[k] = inv @ U[k]
        dp[k] = inv @ rr
    x = np.zeros_like(r)
    for k in range(n - 1, -1, -1):
        x[k] = dp[k] - (C[k] @ x[k + 1] if k + 1 < n else 0)
    return x.astype(np.float64), used


def _matvec(D, U, x, shifts):
    y = np.einsum("nij,nj->ni", D, x) + shifts[:, None] * x
    y[:-1] += np.einsum("nij,nj->ni", U[:-1], x[1:])
    y[1:] += np.einsum("nji,nj->ni", U[:-1], x[:-1])
    return y


def _scaled_solver(D, U, shifts):
    """FP32 block Thomas of the symmetrically scaled system."""
    sv = 1.0 / np.sqrt(np.abs(np.einsum("nii->ni", D) + shifts[:, None]))
    Ds = D * sv[:, :, None] * sv[:, None, :]
    Us = U * sv[:, :, None] * np.roll(sv, -1, axis=0)[:, None, :]
    eye = np.eye(6)

    def solve(b):
        # Scaled shifts: the diagonal shift enters D before scaling.
        Dss = Ds + shifts[:, None, None] * eye[None] * (sv[:, :, None] * sv[:, None, :])
        x, _ = _thomas(Dss, Us, b * sv, np.float32, shifts=np.zeros(len(D)))
        return x * sv
    return solve


def test_fp32_block_factorization_cannot_be_refined(oracle_lib):
    lib = oracle_lib
    sc = scenes.ellipsoid_scene(strands=30, frames=2)
    s = kn.HairSolver(lib)
    scenes.load_into(s, sc)
    lib.lib.khsOracleSetSubstepLimit(ctypes.c_uint32(1))
    try:
        s.step_animation_frame(1, sc.frame_dt)
    finally:
        lib.lib.khsOracleSetSubstepLimit(ctypes.c_uint32(0))
    N = lib.khsGetInternalNodeCount(s.handle)
    S = sc.strands
    diag = np.zeros((N, 6, 6)); upper = np.zeros((N, 6, 6)); g = np.zeros((N, 6)); st = np.zeros((S, 3), np.uint32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    lib.lib.khsOracleExportSystem(s.handle, P(diag), P(upper), P(g), P(st))
    s.close()
    res = {k: [] for k in ("fp64", "fp32", "fp32_refined", "scaled", "scaled_refined")}
    for first, count, fixed in st:
        b, e = int(first + fixed), int(first + count)
        if e - b < 4:
            continue
        D, U, rhs = diag[b:e], upper[b:e], -g[b:e]
        x64, shifts = _thomas(D, U, rhs, np.float64)
        norm = np.linalg.norm(rhs)
        rel = lambda x: np.linalg.norm(rhs - _matvec(D, U, x, shifts)) / norm
        res["fp64"].append(rel(x64))
        f32 = lambda r: _thomas(D, U, r, np.float32, shifts=shifts)[0]
        sc32 = _scaled_solver(D, U, shifts)
        for name, solve in (("fp32", f32), ("scaled", sc32)):
            x = solve(rhs)
            res[name].append(rel(x))
            for _ in range(3):
                x = x + solve(rhs - _matvec(D, U, x, shifts))
            res[name + "_refined"].append(rel(x))
    med = {k: float(np.median(v)) for k, v in res.items()}
    print("median relative residual: " + "  ".join(f"{k} {v:.2e}" for k, v in med.items()))
    assert med["fp64"] < 1e-6               # FP64 direct solve: accurate to the conditioning
    assert med["fp32"] > 1e-2               # the FP32 factorisation is not a usable solve
    assert med["fp32_refined"] > 1e-2       # and FP64 refinement does not recover it
    assert med["scaled"] > 1e-2             # diagonal scaling does not rescue it
    assert med["scaled_refined"] > 1e-2     # not even with refinement
