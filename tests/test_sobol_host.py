"""The raw-sample draw's algorithm on the host: point k of torch's scrambled
SobolEngine is the digital shift XOR the direction numbers selected by the bits
of the Gray code of k, times 2^-maxbit (point 0 as the engine returns it) --
what the device kernel (botorch_gb300/csrc/sobol.cu) computes. Checked bit for
bit against the engine, the sequence the reference's draw_sobol_samples uses
(botorch/utils/sampling.py:74-111)."""

import numpy as np
import pytest
import torch


def gray_code_points(engine: torch.quasirandom.SobolEngine, n: int) -> np.ndarray:
    st = engine.sobolstate.numpy()
    sh = engine.shift.numpy()
    out = np.empty((n, engine.dimension))
    out[0] = engine._first_point.to(torch.float64).numpy()[0]
    for k in range(1, n):
        g, v, b = k ^ (k >> 1), sh.copy(), 0
        while g:
            if g & 1:
                v ^= st[:, b]
            g >>= 1
            b += 1
        out[k] = v.astype(np.float64) * (1.0 / (1 << engine.MAXBIT))
    return out


@pytest.mark.parametrize("dim,n,seed", [(800, 300, 0), (7, 1000, 5), (1, 2, 3)])
def test_gray_code_restatement_matches_the_engine(dim, n, seed):
    ref = torch.quasirandom.SobolEngine(dim, scramble=True, seed=seed).draw(n, dtype=torch.float64).numpy()
    mine = gray_code_points(torch.quasirandom.SobolEngine(dim, scramble=True, seed=seed), n)
    assert np.array_equal(mine, ref)
