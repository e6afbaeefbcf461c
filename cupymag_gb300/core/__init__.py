"""Parameters, config loading, operator setup and the LLG driver."""
