% BUILD_MEX builds the MATLAB gateways of the GB300 f(A)b engine.
% Run from this directory after building ../_lib/libgpumatfun.so
% (python -c "import __graft_entry__ as g; g.build()" at the repository root).
% The gateway names are those lanczosEngine.m calls, so the reference's
% MATLAB scripts run unchanged against this engine.
lib = fullfile('..', '_lib');
names = {'lanczos_create', 'lanczos_delete', 'build_subspace_mex', 'lin_sys_solves_mex', ...
         'apply_V_mex', 'update_U_mex', 'update_U_monodomain_mex', 'get_U_mex', 'get_xsol_mex', ...
         'get_aabb_mex', 'set_y_mex', 'get_basis_mex', 'get_ode_mex', 'set_state_mex', 'solve_mex', 'time_loop_mex', 'fe_create_mex', 'fe_forward_mex', 'fe_backward_mex', 'deflation_pairs_mex'};
for i = 1:numel(names)
    mex('-largeArrayDims', [names{i} '.cpp'], ['-L' lib], '-lgpumatfun', ['LDFLAGS=$LDFLAGS -Wl,-rpath,' lib]);
end
