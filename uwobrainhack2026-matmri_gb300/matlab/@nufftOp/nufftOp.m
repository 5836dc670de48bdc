classdef nufftOp
    % Drop-in for operators/@nufftOp (nufftOp.m:1-136): same constructor
    % N = nufftOp(imN, kloc, dcf, useGPU, os, kwidth), same N*x / N'*y, backed
    % by libmatmri_gb300 (GB300, complex single; double in -> double out).
    % Host arrays and gpuArrays are both accepted (nufftOp.m:335-347); a
    % gpuArray input gives a gpuArray result without a host copy.
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
        tos = [];
        tkwidth = [];
        h = [];          % mmrHandle shared by copies (N and N' share one plan)
        dcf_ = [];
    end
    methods
        function obj = nufftOp(imN, kloc, dcf, useGPU, os, kwidth)
            if nargin < 1
                % no inputs: run the self-tests, as the reference does (nufftOp.m:90-93)
                obj.tests();
                return;
            end
            if nargin > 2 && ~isempty(dcf), obj.dcf_ = double(dcf(:)); end
            if nargin > 3 && ~isempty(useGPU), obj.useGPU = useGPU; end
            if nargin > 4 && ~isempty(os), obj.os = os; end
            if nargin > 5 && ~isempty(kwidth), obj.kwidth = kwidth; end
            obj.imgN = imN;
            obj.kloc = double(kloc);
            obj.h = obj.newPlan();
        end
        function v = get.dcf(obj)
            v = obj.dcf_;
        end
        function obj = set.dcf(obj, v)
            % dcf is a value property (nufftOp.m:70): this copy gets its own plan with the new
            % weights, so that other copies (N', an earlier N) keep theirs
            obj.dcf_ = double(v(:));
            obj.h = obj.newPlan();
            if obj.isToep
                matmri_mex('nufft_prep_toep', obj.h.ptr, obj.tos, obj.tkwidth);
            end
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
            onGPU = isa(x, 'gpuArray');
            if onGPU
                wasDouble = strcmp(classUnderlying(x), 'double');
                x = complex(single(x));                          % converted on the GPU
            end
            y = matmri_mex('nufft_apply', obj.h.ptr, double(obj.adjoint && ~obj.isToep), x, outDims, prod(extra));
            if onGPU && wasDouble, y = double(y); end
        end
        function obj = prepToep(obj, tos, kwidth)
            if obj.isToep, return; end
            if nargin < 2, tos = []; end
            if nargin < 3, kwidth = []; end
            obj.h = obj.newPlan();                               % own plan (value semantics)
            matmri_mex('nufft_prep_toep', obj.h.ptr, tos, kwidth);
            obj.tos = tos;
            obj.tkwidth = kwidth;
            obj.isToep = true;
            obj.loopDim = obj.loopDim + 1;
        end
    end
    methods (Access = private)
        function hh = newPlan(obj)
            hh = mmrHandle(matmri_mex('nufft_create', double(obj.imgN), obj.kloc, obj.dcf_, obj.os, obj.kwidth), 'nufft');
        end
    end
    methods (Static, Access = private)
        function tests()
            % The reference's own identities (@nufftOp/tests.m:30-37, 90-101) on this backend,
            % with thresholds for complex single arithmetic.
            rng(1);
            imN = [24 20];
            kloc = rand(500, 2) - 0.5;
            N = nufftOp(imN, kloc, [], 1, 2, 4);
            x = complex(randn([imN 2]), randn([imN 2]));
            y = complex(randn(500, 2), randn(500, 2));
            lhs = sum(reshape(conj(N*x) .* y, [], 1));
            rhs = sum(reshape(conj(x) .* (N'*y), [], 1));
            assert(abs(lhs - rhs) / abs(lhs) < 1e-5, 'nufftOp adjoint test failed');
            % Cartesian sampling equals the centered FFT (unitary)
            [k1, k2] = ndgrid((-imN(1)/2:imN(1)/2-1)/imN(1), (-imN(2)/2:imN(2)/2-1)/imN(2));
            N = nufftOp(imN, [k1(:) k2(:)], [], 1, 2, 6);
            xc = complex(randn(imN), randn(imN));
            f = fftshift(fft2(ifftshift(xc))) / sqrt(prod(imN));
            d = N * xc;
            phs = d(:) ./ f(:);
            assert(norm(d(:) - mean(phs) * f(:)) / norm(f(:)) < 1e-4, 'nufftOp Cartesian test failed');
            fprintf('nufftOp (GB300) self-tests passed\n');
        end
    end
end
