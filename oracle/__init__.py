"""CPU oracle (test infrastructure only): a NumPy restatement of the reference
single-site TDVP / DMRG path, pinned by the golden fixtures in tests/golden/.
Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may import it."""
