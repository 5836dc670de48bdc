function [x, resSqAll, mseAll, xnormAll, xdiffAll, stopThresh, status] = cgne(Ain, bin, x0, NitMax, opt, gam, Rin, W)
% Drop-in for iterativeSolvers/cgne.m (same arguments and outputs).  The whole
% solve runs on the GB300 (matmri_mex 'cgne'): A is a GB300 nufftOp /
% sampHighOrder, or opFunc = @(x,transp) mrSampFunc(x,transp,S,R[,opt]) over
% GB300 operators, in which case the mrSampFunc options opt.W and opt.tikReg
% (scalar) and the vectorisation options opt.imNFull / opt.daNFull are honoured.
% Tikhonov terms gam / Rin (cgne.m:171-179) are supported for elementwise R
% (numeric scalars or arrays, one per gam in a cell).  Anything else raises
% matmri:gb300:unsupported: there is no host fallback.
if nargin < 3, x0 = []; end
if nargin < 4 || isempty(NitMax), NitMax = 1000; end
if nargin < 5 || isempty(opt), opt = struct(); end
if nargin < 6, gam = []; end
if nargin < 7, Rin = []; end
if nargin < 8, W = []; end
unsupported = @(msg) error('matmri:gb300:unsupported', 'cgne on the GB300: %s', msg);

% ---- the operators: an object, or the variables an mrSampFunc handle captured
S = []; R = []; sopt = struct();
if isa(Ain, 'function_handle')
    fi = functions(Ain);
    if ~contains(fi.function, 'mrSampFunc')
        unsupported('A must be @(x,transp) mrSampFunc(x,transp,S,R[,opt]) over GB300 operators');
    end
    if isfield(fi, 'workspace') && ~isempty(fi.workspace)
        vars = fi.workspace{1};
        names = fieldnames(vars);
        for k = 1:numel(names)
            v = vars.(names{k});
            if isa(v, 'nufftOp') || isa(v, 'sampHighOrder'), S = v; end
            if isa(v, 'rcvrOp'), R = v; end
            if isstruct(v) && any(isfield(v, {'W', 'tikReg', 'imNFull', 'daNFull', 'sumDims', 'hardReal'}))
                sopt = v;
            end
        end
    end
elseif isa(Ain, 'nufftOp') || isa(Ain, 'sampHighOrder')
    S = Ain;
end
if isempty(S) || ~isprop(S, 'h')
    unsupported('no GB300 nufftOp / sampHighOrder found in A');
end
if isa(S, 'nufftOp') && S.isToep
    unsupported('mrSampFunc over a Toeplitz nufftOp applies N''N in both directions');
end
if isfield(sopt, 'sumDims') && ~isempty(sopt.sumDims), unsupported('opt.sumDims'); end
if isfield(sopt, 'hardReal') && ~isempty(sopt.hardReal) && sopt.hardReal, unsupported('opt.hardReal'); end
senseW = []; tikReg = 0;
if isfield(sopt, 'W'), senseW = sopt.W; end
if isfield(sopt, 'tikReg') && ~isempty(sopt.tikReg)
    if numel(sopt.tikReg) ~= 1, unsupported('opt.tikReg with separate real / imaginary weights'); end
    tikReg = double(sopt.tikReg);
end
vecOut = isfield(sopt, 'imNFull') && ~isempty(sopt.imNFull);

% ---- Tikhonov terms sum_k gam_k R_k' R_k for elementwise R_k (cgne.m:91-96, 171-179)
if ~isempty(gam) && ~iscell(gam) && all(gam(:) == 0), gam = []; end
tikDiag = [];
if ~isempty(gam)
    if isempty(Rin), error('cgne: gam needs R'); end
    if ~iscell(gam), gam = {gam}; Rin = {Rin}; end
    if ~iscell(Rin) || numel(Rin) ~= numel(gam), error('cgne: gam and R must match'); end
    tikDiag = 0;
    for k = 1:numel(gam)
        if ~isnumeric(Rin{k}) || ~isnumeric(gam{k}) || numel(gam{k}) ~= 1
            unsupported('Tikhonov operators other than elementwise arrays with scalar gam');
        end
        tikDiag = tikDiag + double(gam{k}) * abs(double(gather(Rin{k}))).^2;
    end
end

% ---- the device solve
if isa(S, 'nufftOp')
    hn = S.h.ptr; hs = uint64(0); imDims = S.imgN; M = size(S.kloc, 1);
else
    hn = uint64(0); hs = S.h.ptr; imDims = S.imSize; M = prod(S.kSize);
end
if isempty(R), hr = uint64(0); else, hr = R.h.ptr; end
if ~isempty(tikDiag) && numel(tikDiag) == 1, tikDiag = repmat(tikDiag, [imDims 1]); end
if ~isempty(tikDiag) && numel(tikDiag) ~= prod(imDims), unsupported('R must be a scalar or an image-sized array'); end
onGPU = isa(bin, 'gpuArray');
wasDouble = strcmp(class(bin), 'double') || (onGPU && strcmp(classUnderlying(bin), 'double'));
if onGPU
    bin = complex(single(bin));
    if ~isempty(x0), x0 = complex(single(x0)); end
end
nda = numel(bin);
if tikReg ~= 0 && isfield(sopt, 'daNFull') && ~isempty(sopt.daNFull)
    nda = prod(sopt.daNFull);                % data rows of the Tikhonov-stacked vector (mrSampFunc.m:121-125)
    tail = bin(nda+1:end);
    if any(tail(:) ~= 0), unsupported('opt.tikReg with non-zero stacked Tikhonov rows in b'); end
    bin = bin(1:nda);
end
[x, resSqAll, mseAll, xnormAll, xdiffAll, stopThresh, status] = matmri_mex('cgne', hn, hs, hr, bin, x0, NitMax, ...
    opt, W, imDims, tikDiag, senseW, tikReg, double(numel(senseW) > M));
if onGPU && wasDouble, x = double(x); end
if vecOut, x = x(:); end
end
