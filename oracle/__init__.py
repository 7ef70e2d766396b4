"""CPU oracle of the GB300 LP solver — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this package, as the checker (or the timed CPU baseline); the product never
imports it.

  ref      ctypes binding of cpu_ref.c (plain-C restatement of the reference
           method, bit-identical to the FP64 GPU kernel)
  exact    exact rational dense simplex (fractions.Fraction), small LPs
  glpk     GLPK 4.45 from the reference's lib/ (x86 container only)
"""
