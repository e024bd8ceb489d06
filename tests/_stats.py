"""Statistical image comparison used by the renderer parity tests.

Two Monte Carlo estimators of the same image are compared through several independent runs of
each: with per-pixel sample variances s_a^2, s_b^2 over the runs, the expected mean squared
difference of the run means is E = mean(s_a^2 / n_a + s_b^2 / n_b).  An unbiased pair gives
MSE / E close to 1; a bias adds its square.  The image means must also agree within 4 standard
errors."""
import numpy as np


def compare_runs(runs_a, runs_b, max_ratio=1.5, n_se=4.0):
    A = np.asarray(runs_a, np.float64)[..., :3]
    B = np.asarray(runs_b, np.float64)[..., :3]
    na, nb = len(A), len(B)
    ma, mb = A.mean(0), B.mean(0)
    va = A.var(0, ddof=1) / na
    vb = B.var(0, ddof=1) / nb
    expected = float(np.mean(va + vb))
    mse = float(np.mean((ma - mb) ** 2))
    se = float(np.sqrt(np.sum(va + vb)) / ma.size)
    dm = float(ma.mean() - mb.mean())
    assert mse <= max_ratio * expected, f"MSE {mse:.3e} > {max_ratio} x expected {expected:.3e}"
    assert abs(dm) <= n_se * se + 1e-7, f"image means differ by {dm:.3e} (SE {se:.3e})"
    return mse / expected, dm / max(se, 1e-12)
