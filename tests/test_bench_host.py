"""Host-side pieces of bench.py that need no GPU: the oracle-check runner."""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def test_run_checks_phases_and_errors():
    import bench
    order = []

    def two_phase(threads):
        order.append(("mt", threads))
        yield
        order.append("seq")
        return {"exact_vs_oracle": True}

    def no_yield(threads):
        return {"exact_vs_oracle": True, "direct": True}
        yield   # makes this a generator function

    def fails(threads):
        yield
        raise ValueError("planted")

    out = bench.run_checks({"a": two_phase, "b": no_yield, "c": fails})
    assert out["a"] == {"exact_vs_oracle": True}
    assert out["b"]["direct"] is True
    assert out["c"]["exact_vs_oracle"] is False and "planted" in out["c"]["error"]
    assert order[0][0] == "mt" and order[0][1] >= 1 and order[-1] == "seq"
