"""CPU oracle for the flare++ prediction path.

TEST INFRASTRUCTURE ONLY.  Nothing in the ``flare_pp_gb300`` package imports
this package; only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it, and only as
the checker or as the timed CPU baseline, never as the thing measured.

The modules restate, in FP64 numpy (and in plain C under ``oracle/c``), the
algorithms of mir-group/flare_pp that sit on the prediction hot path:

* ``geometry``  -- ``Structure`` (src/flare_pp/structure.cpp:27-165)
* ``basis``     -- chebyshev radial basis, cutoff functions, real spherical
                   harmonics (src/flare_pp/radial.cpp:138-169,344-379,
                   src/flare_pp/cutoffs.cpp:44-73, src/flare_pp/y_grad.cpp:667)
* ``b2``        -- B2 descriptor and DescriptorValues
                   (src/flare_pp/descriptors/b2.cpp:76-399)
* ``kernel``    -- NormalizedDotProduct
                   (src/flare_pp/kernels/normalized_dot_product.cpp)
* ``sparse_gp`` -- SparseGP training solve and prediction
                   (src/flare_pp/bffs/sparse_gp.cpp:135-702)
* ``pair_flare``-- mapped-beta pair style
                   (lammps_plugins/pair_flare.cpp:68-396,
                   lammps_plugins/lammps_descriptor.cpp:7-304)

Parity pinning: the reference's own ``radial.cpp``, ``cutoffs.cpp`` and
``y_grad.cpp`` compile unmodified; ``oracle/ref/build_ref.sh`` builds them into
``oracle/_ref/libflare_ref.so`` and ``tests/golden/make_golden.py`` records
their outputs as golden vectors that the oracle is tested against.  The rest
of the reference (structure, b2, kernels, sparse GP, pair style) needs Eigen
and nlohmann_json, which are not available, so those parts are pinned by the
reference's own self-consistency tests (finite differences, sum rules,
beta-form versus kernel-form equality) restated in ``tests/``.
"""
