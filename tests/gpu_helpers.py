"""Helpers for the GPU parity tests: build solvers / problems from fixtures."""
SOLVER_ARRAYS = ('uvw', 'antenna1', 'antenna2', 'frequency', 'ref_frequency', 'parallactic_angles',
                 'point_errors', 'antenna_scaling', 'E_beam', 'G_term', 'lm', 'stokes', 'alpha',
                 'gauss_shape', 'sersic_shape', 'flag', 'weight_vector', 'observed_vis')
PROPS = ('gauss_scale', 'two_pi_over_c', 'sigma_sqrd', 'beam_ll', 'beam_lm', 'beam_lfreq',
         'beam_ul', 'beam_um', 'beam_ufreq')

# Tolerances: max |a-b| / max |b|.  FP64 is the 1e-10 bar; FP32 follows the
# reference's float tests (rtol 1e-3 on chi^2 terms, 1e-4 on the beam).
TOL = {'double': {'vis': 1e-10, 'terms': 1e-10, 'X2': 1e-10, 'jones': 1e-10, 'bsqrt': 1e-12},
       'float': {'vis': 2e-5, 'terms': 1e-3, 'X2': 1e-4, 'jones': 2e-5, 'bsqrt': 2e-6}}


def solver_for(P, dtype, pipeline, extra=None):
    import montblanc_gb300 as mb
    ntime, na = P['uvw'].shape[:2]
    cfg = mb.rime_solver_cfg(
        ntime=ntime, na=na, nchan=P['frequency'].shape[0], nbl=P['antenna1'].shape[1],
        sources=mb.sources(point=P['npsrc'], gaussian=P['ngsrc'], sersic=P['nssrc']),
        beam_lw=P['E_beam'].shape[0], beam_mh=P['E_beam'].shape[1], beam_nud=P['E_beam'].shape[2],
        weight_vector=bool(P['use_weight_vector']),
        vis_output='residuals' if P['residuals'] else 'model',
        dtype=dtype, data_source='empty', pipeline=pipeline, **(extra or {}))
    s = mb.rime_solver(cfg)
    for n in SOLVER_ARRAYS:
        getattr(s, 'transfer_' + n)(P[n])
    for n in PROPS:
        getattr(s, 'set_' + n)(P[n])
    return s
