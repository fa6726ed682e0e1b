"""CPU oracle of the assembly path: test infrastructure only (the parity checker and the timed CPU baseline).
Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import it; the product never does."""
