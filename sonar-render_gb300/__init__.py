"""GB300-native discrete Kirchhoff / Green's-function integration (sonar-render hot path).

Modules:
  api     ctypes binding of the C-ABI library (build/libsonar_gb300.so), named
          like the reference's run_scripts/modules/api.py
  scenes  numpy scene generators and the benchmark workloads
  build   nvcc/g++ build recipe of the library (sm_103a)

The directory name contains a hyphen, so load it as a package with
``__graft_entry__.load_package()`` (or importlib with this file's path).
"""
