"""Command lines: slemm (C++, slemm.cpp) and the GWAS step-2 commands slemm_gamma and slemm_gwa."""
