"""CPU oracle for the rule-based blocking hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline and
reference legs import this package, and only to check the engine's results or
as the timed CPU baseline.  The product (``hyperblocker_gb300``) never imports it.

Contents
--------
``hbx_oracle.cpp``  C++ restatement of the reference's partitioner, plan
                    interpreter, equality, Jaro and Jaro-Winkler
                    (core/components/data_mngr.h, core/gpu/global_func.cuh,
                    core/gpu/device_func.cuh), run as the reference runs it:
                    a brute-force loop over every pair of every partition.
``ref/``            recipe that compiles the reference's own kernel headers for
                    the CPU (``oracle/_ref/libhb_ref.so``, built only where the
                    reference checkout exists) to pin the restatement.
``csvref.py``       the CSV tokenizer of rapidcsv (the reference's CSV
                    dependency, data_mngr.h:48-51), restated.
``rules.py``        YAML rule decoding and plan serialisation
                    (core/common/yaml_config.h, execution_plan_generator.h).
``api.py``          ctypes bindings and the end-to-end oracle run.
"""
