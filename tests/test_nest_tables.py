"""Host logic of the nested chain, on the CPU: nested.nest_tables (the
NestedGrid.f:104-148 tables with pinpoint) equals the oracle's tables for the
children of the nested workload, and a child outside its parent is refused
as NestedGrid.f refuses it."""
import importlib

import numpy as np
import pytest

import oracle

nested = importlib.import_module("cliffs-src_gb300.nested")


@pytest.mark.parametrize("scale", ["small", "full"])
def test_nest_tables_match_oracle(scale):
    if scale == "small":
        levels, _ = nested.SMALL()
    else:
        levels, _ = nested.pkg.workloads.nested_sphere(perturb=0.0, ngauges=1)
    for a, b in zip(levels, levels[1:]):
        got = nested.nest_tables(a["xcrd"], a["ycrd"], b["xcrd"], b["ycrd"])
        ref = oracle.NestTables(a["xcrd"], a["ycrd"], b["xcrd"], b["ycrd"]).as_dict()
        for k, v in ref.items():
            assert np.array_equal(np.asarray(got[k]), np.asarray(v)), k


def test_child_outside_parent_refused():
    x = np.linspace(0.0, 10.0, 11)
    with pytest.raises(ValueError):
        nested.nest_tables(x, x, np.linspace(5.0, 10.5, 12), np.linspace(2.0, 4.0, 5))
