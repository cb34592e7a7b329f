"""CPU oracle of the FSIG matching path: test infrastructure only (the checker,
never the product).  Importable by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py."""
