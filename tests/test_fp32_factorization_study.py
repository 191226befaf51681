"""Why the mixed form keeps the block factorisation in FP64.

Takes real Gauss-Newton systems of the oracle (contact scene, first substeps)
and solves every strand's block-tridiagonal system three ways:
FP64 block Thomas, FP32 block Thomas, and FP32 block Thomas followed by FP64
iterative refinement (r = -g - H x in FP64, x += FP32 solve of r), with and
without symmetric diagonal scaling.  The systems are ill-conditioned (tiny
rotational inertia against stiff stretch/shear), so the FP32 factorisation's
relative residual is O(1) and refinement diverges -- an FP32 factorisation
cannot recover the FP64 direction.  Small CPU case; runs the oracle only.
"""
import ctypes

import numpy as np

import khs_native as kn
import scenes


def _thomas(D, U, rhs, dtype):
    n = len(D)
    D = D.astype(dtype); U = U.astype(dtype); r = rhs.astype(dtype)
    C = np.zeros_like(D); dp = np.zeros_like(r)
    for k in range(n):
        B = D[k].copy(); rr = r[k].copy()
        if k > 0:
            B -= U[k - 1].T @ C[k - 1]
            rr -= U[k - 1].T @ dp[k - 1]
        inv = np.linalg.inv(B)
        if k + 1 < n:
            C[k] = inv @ U[k]
        dp[k] = inv @ rr
    x = np.zeros_like(r)
    for k in range(n - 1, -1, -1):
        x[k] = dp[k] - (C[k] @ x[k + 1] if k + 1 < n else 0)
    return x.astype(np.float64)


def _scaled(D, U, rhs, dtype):
    sv = 1.0 / np.sqrt(np.abs(np.einsum("nii->ni", D)))
    Ds = D * sv[:, :, None] * sv[:, None, :]
    Us = U * sv[:, :, None] * np.roll(sv, -1, axis=0)[:, None, :]
    return _thomas(Ds, Us, rhs * sv, dtype) * sv


def _matvec(D, U, x):
    y = np.einsum("nij,nj->ni", D, x)
    y[:-1] += np.einsum("nij,nj->ni", U[:-1], x[1:])
    y[1:] += np.einsum("nji,nj->ni", U[:-1], x[:-1])
    return y


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
    fp64, fp32, refined, scaled = [], [], [], []
    for first, count, fixed in st:
        b, e = int(first + fixed), int(first + count)
        if e - b < 4:
            continue
        D, U, rhs = diag[b:e], upper[b:e], -g[b:e]
        norm = np.linalg.norm(rhs)
        rel = lambda x: np.linalg.norm(rhs - _matvec(D, U, x)) / norm
        fp64.append(rel(_thomas(D, U, rhs, np.float64)))
        x = _thomas(D, U, rhs, np.float32)
        fp32.append(rel(x))
        for _ in range(3):
            x = x + _thomas(D, U, rhs - _matvec(D, U, x), np.float32)
        refined.append(rel(x))
        scaled.append(rel(_scaled(D, U, rhs, np.float32)))
    fp64, fp32, refined, scaled = map(np.array, (fp64, fp32, refined, scaled))
    print(f"median relative residual: fp64 {np.median(fp64):.2e}  fp32 {np.median(fp32):.2e}  "
          f"fp32+3 refinements {np.median(refined):.2e}  fp32 scaled {np.median(scaled):.2e}")
    assert np.median(fp64) < 1e-6          # FP64 direct solve: accurate to the conditioning
    assert np.median(fp32) > 1e-2          # the FP32 factorisation is not a usable solve
    assert np.median(refined) > np.median(fp32)   # and FP64 refinement diverges from it
    assert np.median(scaled) > 1e-2        # diagonal scaling does not rescue it
