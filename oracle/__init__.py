"""CPU oracle of the reference's SPH fluid step — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this package. The product path (computer_graphics_lab_00_gb300) never
does.
"""
