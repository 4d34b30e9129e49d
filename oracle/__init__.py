"""CPU oracle of rLIC's convolution, and the numpy definition of histogram
equalization (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this package, to check or time the CUDA path; the product
package ``rlic_gb300`` never imports it.
"""
