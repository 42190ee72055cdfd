"""CPU oracle for ProteinSim2015's Langevin step -- TEST INFRASTRUCTURE ONLY.

``oracle.port`` wraps the C restatement (oracle/psim_oracle.c); ``oracle.ref``
wraps the reference itself rebuilt from its sources (oracle/build_ref.sh,
present only where the reference tree is).  Only tests/, the smoke check and
bench.py's CPU legs import this package; the product library never does.
"""
