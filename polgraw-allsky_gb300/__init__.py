"""polgraw_gb300: GB300-native coherent F-statistic search (drop-in for the
Polgraw all-sky network search's job_core hot path).

The directory name contains a hyphen, so the package is registered under the
import name ``polgraw_gb300`` by a path loader (see ``load_package`` in
``bench.py``/``tests/conftest.py``).  Submodules:

* ``lib``   -- ctypes binding of the C-ABI in include/polgraw_gb300.h
* ``build`` -- nvcc/gcc recipes for libpolgraw_gb300.so and the C host
* ``synth`` -- synthetic inputs in the reference's on-disk layout
* ``workloads`` -- the benchmark's synthetic workloads (network, precision
               stress, segments, followup, coincidences)
* ``shards`` -- the sky partitioned over GPUs under torchrun, and the
               reduction of the ranks' timings

The reference host set-up itself (settings, data reading, injection,
ranges) is C, in host/pa_host.c; ``lib.Host`` binds it.
"""
