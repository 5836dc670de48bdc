classdef nufftOp
    % Drop-in for operators/@nufftOp (nufftOp.m:1-136): same constructor
    % N = nufftOp(imN, kloc, dcf, useGPU, os, kwidth), same N*x / N'*y, backed
    % by libmatmri_gb300 (GB300, complex single; double in -> double out).
    properties
        kwidth = 6;
        os = 1.5;
        useGPU = 1;
        useSingle = 0;
        loopDim = 4;
    end
    properties (Dependent)
        dcf;
    end
    properties (SetAccess = protected)
        adjoint = 0;
        kloc = [];
        imgN = [];
        isToep = false;
        h = [];          % mmrHandle shared by copies
        dcf_ = [];
    end
    methods
        function obj = nufftOp(imN, kloc, dcf, useGPU, os, kwidth)
            if nargin < 1
                error('nufftOp:tests', 'self-tests live in the repository test suite');
            end
            if nargin > 2 && ~isempty(dcf), obj.dcf_ = double(dcf(:)); end
            if nargin > 3 && ~isempty(useGPU), obj.useGPU = useGPU; end
            if nargin > 4 && ~isempty(os), obj.os = os; end
            if nargin > 5 && ~isempty(kwidth), obj.kwidth = kwidth; end
            obj.imgN = imN;
            obj.kloc = double(kloc);
            obj.h = mmrHandle(matmri_mex('nufft_create', double(imN), obj.kloc, obj.dcf_, obj.os, obj.kwidth), 'nufft');
        end
        function v = get.dcf(obj)
            v = obj.dcf_;
        end
        function obj = set.dcf(obj, v)
            obj.dcf_ = double(v(:));
            matmri_mex('nufft_set_dcf', obj.h.ptr, obj.dcf_);
        end
        function obj = ctranspose(obj)
            obj.adjoint = xor(obj.adjoint, 1);
        end
        function res = transpose(a)
            res = a';
        end
        function y = mtimes(obj, x)
            nd = numel(obj.imgN);
            sz = size(x);
            if obj.isToep || ~obj.adjoint
                extra = sz(nd+1:end);
                if obj.isToep, outDims = [obj.imgN, extra]; else, outDims = [size(obj.kloc,1), extra]; end
            else
                extra = sz(2:end);
                outDims = [obj.imgN, extra];
            end
            if isempty(extra), extra = 1; end
            y = matmri_mex('nufft_apply', obj.h.ptr, double(obj.adjoint && ~obj.isToep), x, outDims, prod(extra));
        end
        function obj = prepToep(obj, tos, kwidth)
            if obj.isToep, return; end
            if nargin < 2, tos = []; end
            if nargin < 3, kwidth = []; end
            S = nufftOp(obj.imgN, obj.kloc, obj.dcf_, obj.useGPU, obj.os, obj.kwidth);   % own plan (value semantics)
            matmri_mex('nufft_prep_toep', S.h.ptr, tos, kwidth);
            obj.h = S.h;
            obj.isToep = true;
            obj.loopDim = obj.loopDim + 1;
        end
    end
end
