"""CPU oracle for the sqaod hot path -- test infrastructure only.

Imported by tests/, __graft_entry__.smoke() and the CPU legs of bench.py;
never by the product package.
"""
