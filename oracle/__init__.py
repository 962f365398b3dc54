"""CPU oracle for the fastxc_gb300 hot path.

TEST INFRASTRUCTURE ONLY. Nothing in the product package imports this
directory; only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it, always
as the checker or the timed CPU baseline, never as the thing measured or
shipped.

Every function restates the reference algorithm (wangkingh/FastXC) in FP64
numpy and cites the reference file:line it follows. Pinning status of each
module is stated in its own header.
"""
