"""The recorded plans that bench.py's reference arm hands to the oracle's CPU
w-gridder (oracle/plans.json) must be the library planner's choices for the
same workloads, so that the CPU baseline grids the same plan as the GPU."""
import pytest

from oracle import make_plans


@pytest.mark.parametrize("name", make_plans.WORKLOADS)
def test_recorded_plan_matches_planner(wgpu_lib, name):
    recorded = make_plans.load(name)
    current = make_plans.product_plan(name)
    for k in make_plans.FIELDS:
        assert recorded[k] == pytest.approx(current[k], rel=1e-12, abs=0), k


def test_reference_arm_loads_no_product_library():
    """The reference arm's imports (bench.run_reference) stay clear of the
    product's ctypes binding."""
    import ast
    import os
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                            "bench.py")).read()
    tree = ast.parse(src)
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "run_reference")
    names = set()
    for node in ast.walk(fn):
        if isinstance(node, ast.ImportFrom):
            names.update(f"{node.module}.{a.name}" for a in node.names)
        elif isinstance(node, ast.Import):
            names.update(a.name for a in node.names)
    assert not any("_lib" in n or "gridder" in n for n in names), names
