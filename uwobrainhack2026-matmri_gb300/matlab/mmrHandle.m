classdef mmrHandle < handle
    % Owns one libmatmri_gb300 handle; destroyed when the last copy of the
    % value-class operator that holds it goes away (so N and N' share a plan).
    properties
        ptr = uint64(0);
        kind = '';
    end
    methods
        function obj = mmrHandle(ptr, kind)
            obj.ptr = ptr;
            obj.kind = kind;
        end
        function delete(obj)
            if obj.ptr ~= 0
                matmri_mex([obj.kind '_destroy'], obj.ptr);
                obj.ptr = uint64(0);
            end
        end
    end
end
