"""The serving loop's HBM budget split over the (system, N) groups (host
logic, aderdg/serving.py Server.split_budget); no GPU."""
from aderdg.serving import Server


def test_budget_split_equal_and_by_demand():
    need = {"a": 10, "b": 40, "c": 5}
    ub = {"a": 100.0, "b": 200.0, "c": 50.0}
    demand = {"a": 3000.0, "b": 9000.0, "c": 0.0}
    eq = Server.split_budget(120000, demand, need, ub, "equal")
    assert eq == {"a": 400, "b": 200, "c": 800}          # 40000 bytes each
    dm = Server.split_budget(120000, demand, need, ub, "demand")
    assert dm == {"a": 300, "b": 450, "c": 5}            # 30000 / 90000 / 0 bytes, c floored at its largest request
    # a budget below the largest requests: every group holds exactly its largest request
    assert Server.split_budget(1, demand, need, ub, "equal") == need
    assert Server.split_budget(1, demand, need, ub, "demand") == need
