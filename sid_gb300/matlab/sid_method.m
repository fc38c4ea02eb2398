function m = sid_method(name)
% SID_METHOD  Projection form used by the libsid shims: sid_method() returns
% the method number the MEX gateway takes, sid_method(name) sets it.  Names:
%   'direct'              FP32 lenslet convolution (the plain path)
%   'spectral_f32'        FP32 lenslet-grid spectra
%   'spectral_i16'        16-bit block-floating-point spectra
%   'spectral_mixed'      16-bit forward, 24-bit float back projection (default)
%   'spectral_mixed_f32'  16-bit forward, FP32 back projection
persistent current
names = {'direct', 'spectral_f32', 'spectral_i16', 'spectral_mixed', 'spectral_mixed_f32'};
if isempty(current), current = 3; end
if nargin > 0
    k = find(strcmp(names, name), 1);
    if isempty(k), error('sid:method', 'unknown projection method ''%s''', name); end
    current = k - 1;
end
m = current;
end
