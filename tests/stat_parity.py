"""Helpers of the statistical parity tests (tests/test_gpu_statistics.py,
tests/test_statistics_cpu.py): instance ensembles, per-arm statistics and
the two-sample comparisons at alpha = 0.01."""
import numpy as np

ALPHA = 0.01


def ladder(R, tmin, tmax):
    ratio = np.exp(1 / (R - 1) * np.log(tmax / tmin))
    return np.array([1 / (tmin * ratio**k) for k in range(R)], np.float32)


def sk(n, seed):
    rng = np.random.default_rng(seed)
    J = np.triu(rng.normal(size=(n, n)) / np.sqrt(n), 1)
    return (J + J.T).astype(np.float32)


def wishart(n, m, seed):
    rng = np.random.default_rng(seed)
    t = rng.choice([-1.0, 1.0], size=n)
    W = rng.normal(size=(m, n))
    W -= np.outer(W @ t / n, t)
    J = (W.T @ W) / n
    np.fill_diagonal(J, 0.0)
    return J.astype(np.float32)


def e64(J, S):
    S = np.asarray(S, np.float64)
    return np.einsum("ri,ij,rj->r", S, J.astype(np.float64), S) / 2


def arm_stats(J, best_e, best_x, final_x, bidx):
    """Per-read best energy (f64 energy of the best state of the chain with
    the lowest best energy) and per-slot final energies [reads, R]."""
    Rd, R, n = final_x.shape
    k = np.asarray(best_e).reshape(Rd, R).argmin(axis=1)
    best = e64(J, np.asarray(best_x).reshape(Rd, R, n)[np.arange(Rd), k])
    fin = e64(J, final_x.reshape(-1, n)).reshape(Rd, R)
    slots = np.take_along_axis(fin, np.asarray(bidx).reshape(Rd, R), axis=1)
    return best, slots


def compare(arms, label):
    """p-values of every pair of arms; prints them."""
    from scipy import stats
    pooled = np.concatenate([a[0] for a in arms.values()])
    target = np.quantile(pooled, 0.25)
    report = {}
    for x, y in (("gpu", "f32"), ("gpu", "f64"), ("f32", "f64")):
        bx, sx = arms[x]
        by, sy = arms[y]
        ks = stats.ks_2samp(bx, by)
        hx, hy = int((bx <= target).sum()), int((by <= target).sum())
        fisher = stats.fisher_exact([[hx, len(bx) - hx], [hy, len(by) - hy]])
        welch = stats.ttest_ind(sx, sy, axis=0, equal_var=False)
        report[x + "/" + y] = (ks.pvalue, fisher.pvalue,
                               float(np.min(welch.pvalue)) * sx.shape[1],
                               hx / len(bx), hy / len(by))
    for k, (pks, pf, pw, px, py) in report.items():
        print(f"{label} {k}: KS p={pks:.3f}, hit rates {px:.3f} / {py:.3f} "
              f"(Fisher p={pf:.3f}), slot means min Bonferroni p="
              f"{min(pw, 1.0):.3f}")
    for name, (best, slots) in arms.items():
        h = int((best <= target).sum())
        lo, hi = wilson(h, len(best))
        se = best.std(ddof=1) / np.sqrt(len(best))
        print(f"{label} {name}: reads {len(best)}, best energy mean "
              f"{best.mean():.4f} +- {1.96 * se:.4f} (95 %), hit rate at "
              f"{target:.4f}: {h / len(best):.3f} [{lo:.3f}, {hi:.3f}], "
              f"slot 0 (coldest) final energy mean {slots[:, 0].mean():.4f}")
    return report


def wilson(k, m, z=1.96):
    """95 % Wilson score interval of a binomial proportion k / m."""
    p = k / m
    d = 1 + z * z / m
    c = (p + z * z / (2 * m)) / d
    r = z * np.sqrt(p * (1 - p) / m + z * z / (4 * m * m)) / d
    return c - r, c + r


def assert_same(report, label):
    for k, (pks, pf, pw, _, _) in report.items():
        assert pks > ALPHA, (label, k, "KS")
        assert pf > ALPHA, (label, k, "hit rate")
        assert pw > ALPHA, (label, k, "slot energies")


