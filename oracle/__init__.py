"""CPU oracle for the SAIGE step-1 GRM / PCG / AI-REML hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library imports, links or
executes this package: only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it, and only
as the checker (or as the timed CPU restatement of the reference's own CPU
path), never as the thing measured for the GPU path.

The oracle restates, in plain numpy (FP64 unless stated) and plain C, the
algorithm of the reference files (paths relative to the reference project):

* ``src/SAIGE/src/SAIGE_fitGLMM_fast.cpp`` ("FIT.cpp"): genotype decode, QC,
  standardisation, GRM diagonal, GRM.x, Sigma operators, PCG, Hutchinson
  trace, coefficients, AI score, tau update.
* ``src/SAIGE/R/SAIGE_fitGLMM_fast.R`` ("FIT.R"): the AI-REML driver
  (``Get_Coef``, ``glmmkin.ai_PCG_Rcpp_Binary``/``_Quantitative``) and the
  variance-ratio estimate.

Pinning: the decode is pinned bit-exactly to PLINK's ``.frq`` of the
reference's ``plinkforGRM_1000samples_10kMarkers`` example; the full fit is
pinned at Monte-Carlo tolerance to the reference's golden ``.rda`` theta
values (the probes come from R's RNG there, from a counter hash here).
"""
