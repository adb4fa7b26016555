"""ORACLE — TEST INFRASTRUCTURE ONLY: the f64 CPU restatement of the reference's
lifting-line path (sb_oracle.hpp), its build recipe (build.py) and ctypes binding
(binding.py). Never imported by the product package."""
