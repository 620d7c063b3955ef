// Host execution shim of the AmgX C API calls the reference makes
// (kernel/solver.cu:118-135, kernel/bubble.cu:1479-1508).  AmgX itself is not
// available; ref_amgx.cpp solves the uploaded CSR system on the host to a
// tight residual instead (the answer of the solve is defined by the matrix).
#pragma once
typedef enum { AMGX_RC_OK = 0, AMGX_RC_BAD_PARAMETERS = 1 } AMGX_RC;
typedef enum { AMGX_mode_dDDI = 8193, AMGX_mode_dFFI = 8194 } AMGX_Mode;
typedef enum { AMGX_SOLVE_SUCCESS = 0, AMGX_SOLVE_FAILED = 1, AMGX_SOLVE_DIVERGED = 2 } AMGX_SOLVE_STATUS;
typedef struct sbref_amgx_config* AMGX_config_handle;
typedef struct sbref_amgx_resources* AMGX_resources_handle;
typedef struct sbref_amgx_matrix* AMGX_matrix_handle;
typedef struct sbref_amgx_vector* AMGX_vector_handle;
typedef struct sbref_amgx_solver* AMGX_solver_handle;
AMGX_RC AMGX_initialize();
AMGX_RC AMGX_initialize_plugins();
AMGX_RC AMGX_finalize();
AMGX_RC AMGX_finalize_plugins();
AMGX_RC AMGX_config_create_from_file(AMGX_config_handle* cfg, const char* path);
AMGX_RC AMGX_config_destroy(AMGX_config_handle cfg);
AMGX_RC AMGX_resources_create(AMGX_resources_handle* rsc, AMGX_config_handle cfg, void* comm,
                              int device_num, const int* devices);
AMGX_RC AMGX_resources_destroy(AMGX_resources_handle rsc);
AMGX_RC AMGX_matrix_create(AMGX_matrix_handle* mtx, AMGX_resources_handle rsc, AMGX_Mode mode);
AMGX_RC AMGX_matrix_destroy(AMGX_matrix_handle mtx);
AMGX_RC AMGX_vector_create(AMGX_vector_handle* vec, AMGX_resources_handle rsc, AMGX_Mode mode);
AMGX_RC AMGX_vector_destroy(AMGX_vector_handle vec);
AMGX_RC AMGX_solver_create(AMGX_solver_handle* slv, AMGX_resources_handle rsc, AMGX_Mode mode,
                           AMGX_config_handle cfg);
AMGX_RC AMGX_solver_destroy(AMGX_solver_handle slv);
AMGX_RC AMGX_vector_upload(AMGX_vector_handle vec, int n, int block_dim, const void* data);
AMGX_RC AMGX_vector_download(AMGX_vector_handle vec, void* data);
AMGX_RC AMGX_matrix_upload_all(AMGX_matrix_handle mtx, int n, int nnz, int block_dimx,
                               int block_dimy, const int* row_ptrs, const int* col_indices,
                               const void* data, const void* diag_data);
AMGX_RC AMGX_solver_setup(AMGX_solver_handle slv, AMGX_matrix_handle mtx);
AMGX_RC AMGX_solver_solve(AMGX_solver_handle slv, AMGX_vector_handle rhs, AMGX_vector_handle sol);
AMGX_RC AMGX_solver_get_status(AMGX_solver_handle slv, AMGX_SOLVE_STATUS* st);
AMGX_RC AMGX_solver_get_iterations_number(AMGX_solver_handle slv, int* n);
