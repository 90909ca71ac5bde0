"""ORACLE (test infrastructure only): CPU restatement of Mat-8.3.1's hot-path
algorithms (liboracle.so) plus, where the reference headers are available,
the reference itself compiled into _ref/libmatref.so.  Only tests, the smoke
check and the benchmark's CPU-baseline leg may import this package."""
