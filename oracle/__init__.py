"""FP64 CPU oracle for the phinfortran NEGF hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the shipped package imports this
directory; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` use it, always as the reference results are compared
with and never as the code under measurement.

The modules restate the reference Fortran (KitchenSong/phinfortran) in numpy,
batched over (omega, q) points but otherwise step for step:

* ``negf``   -- Lopez-Sancho decimation, block RGF sweeps, Caroli trace
                (negf/surface.f90, negf/lesser.f90, tb/surface.f90,
                tb/device.f90).
* ``qe``     -- Quantum-ESPRESSO force-constant reader, supercell layout,
                grids (negf/fc.f90, negf/config.f90, negf/input.f90).
* ``dyn``    -- block D(q) assembly of the tdb branch (negf/dyn.f90).
* ``velmat`` -- mode-resolved transmission (negf/velocity_mat.f90).

Parity pin: the restatement reproduces the reference's committed si-si run
(examples/negf/si-si/output/trans{l,r}_tot.dat); see tests/test_oracle_golden.py.
"""
