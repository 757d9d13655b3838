// common.h -- status codes returned by the plugin lifecycle calls.  The names
// and their order are codeare's (src/common.h:29-63) so that callers that
// compare against them keep working.
#pragma once

namespace codeare {
enum error_code {
    OK,
    ERROR_GENERAL,
    ERROR_UNKNOWN_METHOD,
    FATAL_SYSTEM_CALL,
    LAPACK_WORKSPACE_QUERY_FAILED,
    CG_DID_NOT_CONVERGE,
    CANNOT_LOAD_LIBRARY,
    UNSUPPORTED_DIMENSION,
    UNSUPPORTED_IMAGE_MATRIX,
    ZERO_NODES,
    CGSENSE_ZERO_CHANNELS,
    FILE_ACCESS_FAILED,
    CONTEXT_CONFIGURATION_FAILED,
    CONTEXT_NOT_FOUND,
    MEM_ALLOC_FAILED,
    FILE_OPEN_FAILED,
    FILE_READ_FAILED,
    FILE_WRITE_FAILED,
    NULL_FILE_HANDLE,
    UNIMPLEMENTED_METHOD,
    HDF5_ERROR_FOPEN,
    HDF5_ERROR_FCLOSE,
    HDF5_ERROR_FFLUSH,
    GENERAL_IO_ERROR,
    CONFIG_LOAD_FILE_FAILED,
    WRONG_OR_NO_DATASET,
    CONFIG_MISSING_CHAIN,
    CONFIG_EMPTY_CHAIN,
    NULL_STRATEGY,
    NO_MATRIX_IN_WORKSPACE_BY_NAME,
    WRONG_MATRIX_TYPE
};
}  // namespace codeare
