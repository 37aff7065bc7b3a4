"""GB300 (sm_103a) engine for GisAPR's candidate-scoring path.

Entry points keep the reference's names and conventions:

* gisapr_gb300.pdb2mrc   -- density_from_coords, generate_volume, MovedChainDensity
* gisapr_gb300.search    -- PackedFourierLayout, PackedCTFTorch, PsiGridBank,
                            ParticleFourierPreparer, IntegratedProjector,
                            CorrelationWorkspace, correlate_templates_and_particle,
                            make_result_records
* gisapr_gb300.engine    -- ScoringJob: a job held on the GPU, one call per pose
* gisapr_gb300.tables    -- host tables (STAR rows, local lists, mask, FSC, CTF terms)

All numeric work runs in the in-tree library libgisapr_gb300.so (C ABI in
include/gisapr_gb300.h); there is no CPU fallback.
"""
__version__ = "0.1.0"
