"""The per-check log lines of usbs() and cgal() (host formatting).  CPU only."""
import re

from usbs_gb300 import solver


def test_log_lines_have_the_reference_fields_in_order():
    """usbs()/cgal() per-check lines: the fields and order of the reference's
    prints (solver/usbs.py:514-530, solver/cgal.py:79-88), with primal_obj
    unscaled by SCALE_C * SCALE_X and callback_val printed as given."""
    rec = {"t": 7, "pen_dual_obj": 1.5, "cand_pen_dual_obj": 1.25, "lb_spec_est": 0.5,
           "primal_obj": 8.0, "dual_obj": 3.0, "obj_ub": 4.0, "obj_gap": 1e-3,
           "infeas_gap": 2e-4, "max_infeas": 3e-5}
    line = solver.log_line(rec, 2.0, 2.0, callback_val=None, curr_time=12.5)
    fields = ["t", "curr_time", "pen_dual_obj", "cand_pen_dual_obj", "lb_spec_est", "primal_obj",
              "dual_obj", "primal_obj_ub", "obj_gap", "infeas_gap", "max_infeas", "callback_val"]
    assert re.findall(r"(\w+): ", line) == fields
    vals = dict(re.findall(r"(\w+): (\S+)", line))
    assert vals["t"] == "7" and float(vals["curr_time"]) == 12.5
    assert float(vals["primal_obj"]) == 2.0                   # 8 / (2 * 2)
    assert float(vals["primal_obj_ub"]) == 4.0 and vals["callback_val"] == "None"
    cl = solver.cgal_log_line(rec, 2.0, 2.0, callback_val=5.0, curr_time=1.0)
    assert re.findall(r"(\w+): ", cl) == ["t", "curr_time", "primal_obj", "obj_gap",
                                          "infeas_gap", "max_infeas", "callback_val"]
    assert cl.endswith("callback_val: 5.0")
