"""CPU oracle of the reference PBD step.  Test infrastructure only (see pbd_oracle.c)."""
