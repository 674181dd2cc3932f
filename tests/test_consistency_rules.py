"""Input validation (Auxiliar.py:24-78): the package raises SystemExit with
the reference's message for every invalid input the reference rejects."""
import numpy as np
import pytest

from conftest import load_golden

api = pytest.importorskip("tensorfox_gb300.api")
opts = pytest.importorskip("tensorfox_gb300.options")


def test_consistency_messages_match_reference():
    g = load_golden("consistency")
    for dims, R, o, msg in zip(g["dims"], g["ranks"], g["opts"], g["msgs"]):
        class O:
            pass
        for k, v in eval(str(o)).items():
            setattr(O, k, v)
        op = opts.make_options(O)
        dims, R = eval(str(dims)), eval(str(R))
        if str(msg) == "":
            api.consistency(R, dims, op)
        else:
            with pytest.raises(SystemExit) as ei:
                api.consistency(R, dims, op)
            assert str(ei.value) == str(msg)
