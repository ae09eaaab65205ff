"""Distribution of independent right-hand sides over processes.

``parallel_task`` restates data/parallel/src/parallel.f90:80-135: every rank
gets num_task_total // size tasks and the last (num_task_total % size) ranks
one more; tasks are contiguous blocks in rank order.  Each GPU process solves
its own block (the perturbations are independent, do_stern.f90:199), so no
collective is needed on the data path; results are gathered on the host.
"""
from __future__ import annotations


def parallel_task(num_task_total: int, rank: int, size: int):
    """Return (first_task, last_task, num_task) with 0-based inclusive bounds."""
    if size < 1 or not 0 <= rank < size:
        raise ValueError("invalid rank/size")
    num_task_min = num_task_total // size
    num_remain = num_task_total % size
    last_proc = size - num_remain
    num_task = [num_task_min] * last_proc + [num_task_min + 1] * num_remain
    last = sum(num_task[:rank + 1])
    first = last - num_task[rank]
    return first, last - 1, num_task
