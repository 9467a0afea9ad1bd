"""ORACLE package: test infrastructure only (see glemur_oracle.c)."""
