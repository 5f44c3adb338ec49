"""Host logic of the FP64 escalation of mixed-precision forced solves (forced_sweep and
KSP.solve), on a stand-in pencil that records the calls: a group whose refinement stops
above the bound is factorised again in FP64 and solved with those factors; a group that
meets it is not."""
import numpy as np

from kore_gb300.solver import KSP, forced_sweep


class FakePencil:
    """Records factorisations; the mixed solve of the shifts in `bad` reports a backward
    error of 1e-9, every other solve 1e-15; x = b * (1 for mixed, 2 for fp64)."""

    def __init__(self, n, bad=()):
        self.n, self.bad, self.calls = n, set(bad), []
        self.sigma, self.precision = None, None

    def factor_shifts(self, sigmas, precision):
        self.calls.append(("factor", tuple(np.round(np.asarray(sigmas).imag, 6)), precision))
        self.sigma, self.precision = tuple(np.asarray(sigmas)), precision

    def factor(self, sigma, precision):
        self.factor_shifts([sigma], precision)

    def solve(self, rhs, refine_tol=0.0, stats=False):
        x = rhs * (1.0 if self.precision == "mixed" else 2.0)
        hit = self.precision == "mixed" and any(round(s.imag, 6) in self.bad for s in self.sigma)
        st = {"solve_resid_max": 1e-9 if hit else 1e-15}
        return (x, st) if stats else x


def test_forced_sweep_escalates_only_bad_groups():
    p = FakePencil(5, bad={0.5})
    om = [0.0, 0.25, 0.5, 0.75]
    b = np.arange(5, dtype=complex)
    info = {}
    X, _ = forced_sweep(p, om, b, "mixed", group=2, info=info)
    assert info == {"escalated": 2, "mixed_resid_max": 1e-9}
    assert [c[2] for c in p.calls] == ["mixed", "mixed", "fp64"]
    assert p.calls[2][1] == (0.5, 0.75)
    np.testing.assert_array_equal(X[:, :2], np.repeat(b[:, None], 2, axis=1))
    np.testing.assert_array_equal(X[:, 2:], 2 * np.repeat(b[:, None], 2, axis=1))


def test_forced_sweep_without_escalation():
    p = FakePencil(3, bad={0.5})
    info = {}
    forced_sweep(p, [0.5], np.ones(3), "mixed", escalate_tol=0.0, info=info)
    assert info["escalated"] == 0 and [c[2] for c in p.calls] == ["mixed"]
    p64 = FakePencil(3, bad={0.5})
    forced_sweep(p64, [0.5], np.ones(3), "fp64", info=info)
    assert info["escalated"] == 0 and [c[2] for c in p64.calls] == ["fp64"]


def test_ksp_escalates():
    p = FakePencil(4, bad={0.0})
    k = KSP()
    k.pencil = p   # setOperators takes a real Pencil only
    k.precision = "mixed"
    x = k.solve(np.ones(4, dtype=complex))
    assert k.stats["escalated"] == 1 and np.all(x == 2.0)
    assert [c[2] for c in p.calls] == ["mixed", "fp64"]
