"""ORACLE — test infrastructure only; never imported by the iactrace_gb300 package."""
