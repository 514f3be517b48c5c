"""Admission policy of the solve service (host logic, no GPU)."""
from usbs_gb300.serving import Admission


def test_slots_and_memory_budget():
    adm = Admission(budget_bytes=100, max_slots=2)
    assert adm.admissible(60, False)
    adm.start(60, False)
    assert not adm.admissible(50, False)       # 60 + 50 > 100
    assert adm.admissible(40, False)
    adm.start(40, False)
    assert not adm.admissible(1, False)        # no slot left
    adm.finish(60, False)
    assert adm.admissible(50, False) and adm.running_bytes == 40


def test_small_requests_pass_one_that_does_not_fit():
    adm = Admission(budget_bytes=100, max_slots=4)
    adm.start(70, False)
    queue = [(50, False), (20, False), (10, False)]
    assert adm.pick(queue) == 1


def test_exclusive_request_waits_for_drain_and_holds_the_line():
    adm = Admission(budget_bytes=1000, max_slots=4)
    adm.start(10, False)
    queue = [(100, True), (5, False)]
    assert adm.pick(queue) is None             # exclusive waits; nothing passes it
    adm.finish(10, False)
    assert adm.pick(queue) == 0
    adm.start(100, True)
    assert adm.pick([(5, False)]) is None      # nothing runs beside an exclusive solve
    adm.finish(100, True)
    assert adm.pick([(5, False)]) == 0


def test_request_larger_than_the_budget_never_fits():
    adm = Admission(budget_bytes=100, max_slots=2)
    assert adm.ever_fits(100) and not adm.ever_fits(101)


def test_request_waiting_for_its_warm_start_parent_does_not_block_others():
    adm = Admission(budget_bytes=100, max_slots=4)
    queue = [(10, False, False), (20, False, True)]
    assert adm.pick(queue) == 1
    assert adm.pick([(10, False, True), (20, False, True)]) == 0
