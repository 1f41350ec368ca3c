"""CPU oracle for the CPanel hot path (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import this
package; the product library (cpanel_gb300) never does.
"""
