"""The oracle's FP32 restatement (the parity target of the kernels) against
its FP64 render of the same paths (libm transcendentals, double arithmetic),
on the CPU: per-path radiance and the converged tile of the Cornell room.
This checks the FP32 shading chain (OpenPBR lobes, E_dielectric estimate,
light sampling, MIS) as a whole against double precision."""
import numpy as np

import oracle


def test_fp32_paths_match_fp64_render(cornell):
    _, _, ow = cornell
    px = np.array([[x, y] for y in range(112, 144) for x in range(112, 144)], np.uint32)
    r32, _ = oracle.trace_paths(ow, (256, 256), 8, px, 1, 16)
    r64, _ = oracle.trace_paths(ow, (256, 256), 8, px, 1, 16, precision=64)
    r32, r64 = r32.astype(np.float64).reshape(-1, 3), r64.astype(np.float64).reshape(-1, 3)
    # almost every path takes the same branches: radiance within 1e-4 relative
    close = np.all(np.abs(r32 - r64) <= 1e-4 * np.abs(r64) + 1e-6, axis=1)
    assert close.mean() > 0.99, close.mean()  # measured: every path
    # the converged tile (16 spp): measured 4.4e-7 relative RMSE
    img32 = r32.reshape(16, -1, 3).mean(axis=0)
    img64 = r64.reshape(16, -1, 3).mean(axis=0)
    rmse = np.sqrt(np.mean((img32 - img64) ** 2)) / np.sqrt(np.mean(img64 ** 2))
    assert rmse < 1e-5, rmse
