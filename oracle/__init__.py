"""CPU oracle for the raycaster and the UVF build (test infrastructure only).

Imported by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg as
the checker; the product never imports it.
"""
