"""Oracles for the fastxc_gb300 hot path.

TEST INFRASTRUCTURE ONLY. Nothing in the product package imports this
directory; only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it, always
as the checker or the timed baseline, never as the thing measured or
shipped.

Two oracles live here:
  * the reference's own CUDA kernels, compiled from its sources by
    ``build_ref.py`` (``ref_kernels.cu``) and run on the GPU in the
    reference's host order by ``ref_gpu.py``;
  * an FP64 numpy restatement of the reference algorithm
    (``sac2spec_oracle.py``, ``xc_oracle.py``, ``stack_oracle.py``), each
    function citing the reference file:line it follows; its integer and
    planning parts are pinned bit-exact against the reference's C compiled
    on the CPU (``build_ref.py``, ``ref_xc_shim.cpp``).
"""
