"""ORACLE / TEST INFRASTRUCTURE ONLY: CPU checkers for the snow MPM step.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg. The product (snow_gb300) never imports it.
"""
