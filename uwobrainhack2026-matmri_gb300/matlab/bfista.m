function [x, resSqAll, RxAll, testAll] = bfista(Ain, bin, Rin, lam, x0, NitMax, opt)
% Drop-in for iterativeSolvers/bfista.m (the first four outputs) when A is a
% GB300 operator or @(x,transp) mrSampFunc(x,transp,S,R) over GB300 operators
% and R is dwtND(J, imSize, false, 'db1') (undecimated Haar): the whole solve,
% powermethod included (bfista.m:81-90), runs on the GB300.  lam is a scalar
% or one threshold per wavelet band (waveletObj order).  Anything else raises
% matmri:gb300:unsupported.
if nargin < 5, x0 = []; end
if nargin < 6 || isempty(NitMax), NitMax = 200; end
if nargin < 7 || isempty(opt), opt = struct(); end
unsupported = @(msg) error('matmri:gb300:unsupported', 'bfista on the GB300: %s', msg);
S = []; R = [];
if isa(Ain, 'function_handle')
    fi = functions(Ain);
    if isfield(fi, 'workspace') && ~isempty(fi.workspace)
        vars = fi.workspace{1};
        names = fieldnames(vars);
        for k = 1:numel(names)
            v = vars.(names{k});
            if isa(v, 'nufftOp') || isa(v, 'sampHighOrder'), S = v; end
            if isa(v, 'rcvrOp'), R = v; end
            if isstruct(v), unsupported('mrSampFunc options'); end
        end
    end
elseif isa(Ain, 'nufftOp') || isa(Ain, 'sampHighOrder')
    S = Ain;
end
if isempty(S) || ~isprop(S, 'h'), unsupported('no GB300 nufftOp / sampHighOrder found in A'); end
if ~isa(Rin, 'dwtND') || Rin.decimation || ~strcmp(Rin.family, 'db1')
    unsupported('R must be an undecimated db1 (Haar) dwtND');
end
if isa(S, 'nufftOp')
    hn = S.h.ptr; hs = uint64(0); imDims = S.imgN;
else
    hn = uint64(0); hs = S.h.ptr; imDims = S.imSize;
end
if isempty(R), hr = uint64(0); else, hr = R.h.ptr; end
levels = double(Rin.J(1:numel(imDims)));
onGPU = isa(bin, 'gpuArray');
if onGPU
    bin = complex(single(bin));
    if ~isempty(x0), x0 = complex(single(x0)); end
end
nb = 1;                                     % bands: 1 + sum over levels of (2^(dims decomposed) - 1)
for lv = 1:max(levels), nb = nb + 2^sum(levels >= lv) - 1; end
lam = double(gather(lam(:)));
if numel(lam) == 1, lam = repmat(lam, nb, 1); end
if numel(lam) ~= nb, error('bfista: lam needs 1 or %d entries (one per band)', nb); end
[x, resSqAll, RxAll, testAll] = matmri_mex('bfista', hn, hs, hr, bin, levels, lam, x0, NitMax, opt, imDims);
end
