function forward_model = update_spatial_component(timeseries, sensor_movie, template, opts)
% Drop-in for update_spatial_component.m (same signature): every template
% pixel's regularised NNLS (reg_nnls -> NQP, FP64 active set) in one libsid
% launch, pixels covered by any number of neurons included; the background
% row outside the templates as in the reference.  Returns the sparse
% forward model the reference builds.
if nargin < 4, opts = struct; end
if ~isfield(opts, 'bg_sub'), opts.bg_sub = 1; end
T = gpuArray(single(timeseries));
if isa(sensor_movie, 'uint16') || isa(sensor_movie, 'half'), Y = gpuArray(sensor_movie); else, Y = gpuArray(single(sensor_movie)); end
Fm = sid_mex('spatial_update', T, Y, logical(template), opts);
forward_model = sparse(double(gather(Fm)));
end
