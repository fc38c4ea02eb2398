function forward_model = generate_LFM_library_GPU(recon, centers, neur_id, psf, options)
% Drop-in for generate_LFM_library_GPU.m (same signature): every neuron's
% boxed, component-averaged volume (options.neur_rad, options.axial) is
% forward-projected in one libsid launch on the PSF's resident plan, giving
% the N x prod(options.image_size) single library on the host.  A neuron
% kernel (options.ker_param) is not applied to the library here.
% options.sid_library = 'spectral' uses the tensor-core spectral projector on
% lenslet windows around the boxes (faster; about 1e-5 relative per row)
% instead of the FP32 lenslet taps ('direct', the default).
if nargin < 5, options = struct; end
if isfield(options, 'ker_param')
    error('sid:generate_LFM_library_GPU', 'a neuron kernel (options.ker_param) is not supported by the library launch');
end
vols = cellfun(@(v) gpuArray(single(v)), recon, 'UniformOutput', false);
plan = sid_plan_for(psf.H, [], options.image_size(1), options.image_size(2));
method = 'direct';
if isfield(options, 'sid_library'), method = options.sid_library; end
F = sid_mex('library', plan, vols, double(centers), logical(neur_id), options.neur_rad, options.axial, method);
forward_model = gather(F);
end
