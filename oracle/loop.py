"""Bounded while-loop semantics of the reference (oracle copy, test infrastructure).

Restates ``utils/loop.py:80-115`` (``while_loop``) and its scan variants
``utils/loop.py:21-51``: the body runs at most ``maxiter`` times, the condition
is evaluated on the initial value and after every body (``cond_exp_base == 1``),
or only after geometric blocks of bodies (``cond_exp_base > 1``,
``utils/loop.py:84-98``).
"""
import math


def cond_schedule(maxiter: int, cond_exp_base: float):
    """Block sizes between condition checks (utils/loop.py:86-92)."""
    assert 1.0 <= cond_exp_base <= 2.0
    if cond_exp_base == 1.0:
        return [1] * maxiter
    num = math.ceil(math.log((cond_exp_base - 1) * maxiter - 1) / math.log(cond_exp_base)) + 1
    steps = [int(cond_exp_base ** i) for i in range(int(num))]
    csum, kept = 0, []
    for s in steps:
        csum += s
        if csum >= maxiter:
            continue
        kept.append(s)
    kept.append(maxiter - sum(kept))
    return kept


def while_loop(cond_fun, body_fun, init_val, maxiter, cond_exp_base=1.0):
    val = init_val
    if cond_exp_base == 1.0:
        cond = cond_fun(val)
        for _ in range(maxiter):
            if not cond:
                break
            val = body_fun(val)
            cond = cond_fun(val)
        return val
    cond = cond_fun(val)
    for steps in cond_schedule(maxiter, cond_exp_base):
        if not cond:
            break
        for _ in range(steps):
            val = body_fun(val)
        cond = cond_fun(val)
    return val
