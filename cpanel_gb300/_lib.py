"""ctypes binding of libcpanel_gb300.so (the in-tree CUDA extension).

There is no CPU fallback: if the library is missing or no CUDA device is usable,
calls raise CpgError.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcpanel_gb300.so")

D = C.POINTER(C.c_double)
I32 = C.POINTER(C.c_int32)
I64 = C.POINTER(C.c_int64)
# cpg_velocity_fn: (user, points m x 3, m, velocities m x 3) -> status
VELOCITY_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, D, C.c_int64, D)

STATUS = {0: "CPG_OK", 1: "CPG_E_INVALID", 2: "CPG_E_OOM", 3: "CPG_E_CUDA", 4: "CPG_E_BAD_MESH",
          5: "CPG_E_NOT_CONVERGED", 6: "CPG_E_TIMEOUT", 7: "CPG_E_NO_DEVICE"}
PLAIN_FP64, MIXED = 0, 1


class CpgError(RuntimeError):
    def __init__(self, code, msg=""):
        self.code = code
        super().__init__("%s: %s" % (STATUS.get(code, str(code)), msg))


class GeometryInfo(C.Structure):
    _fields_ = [("n_body", C.c_int64), ("n_wake", C.c_int64), ("n_wakes", C.c_int64), ("n_wakelines", C.c_int64),
                ("n_tip", C.c_int64), ("n_nodes", C.c_int64), ("h2d_bytes", C.c_int64)]


PROF_CLASSES = ["assembly", "wake_columns", "matvec_fp32", "matvec_fp64", "residual", "lu_factor", "particles",
                "chtls", "post", "lu_solve", "tc_gemm"]


class Prof(C.Structure):
    _fields_ = [("launches", C.c_longlong * len(PROF_CLASSES)), ("ms", C.c_double * len(PROF_CLASSES))]


class Flow(C.Structure):
    _fields_ = [("V", C.c_double), ("alpha", C.c_double), ("beta", C.c_double), ("mach", C.c_double)]


class Refs(C.Structure):
    _fields_ = [("Sref", C.c_double), ("bref", C.c_double), ("cref", C.c_double), ("cg", C.c_double * 3)]


class CaseOut(C.Structure):
    _fields_ = [(name, D) for name in ("mu", "sigma", "phi", "vel", "cp", "CL", "CDi", "Fbody", "Fwind", "CM")]


class SolveStats(C.Structure):
    _fields_ = [("iters_max", C.c_int64), ("iters_total", C.c_int64), ("refinements", C.c_int64),
                ("residual_max", C.c_double), ("n_near", C.c_int64), ("n_far", C.c_int64),
                ("ms_assemble", C.c_double), ("ms_solve", C.c_double), ("ms_post", C.c_double)]


_lib = None

# every symbol declared in include/cpanel_gpu.h
EXPORTS = ["cpg_create", "cpg_destroy", "cpg_last_error", "cpg_set_stream", "cpg_synchronize",
           "cpg_geometry_create", "cpg_geometry_destroy", "cpg_geometry_info_get", "cpg_geometry_tables", "cpg_topology",
           "cpg_set_inf_coeff", "cpg_get_A", "cpg_get_B", "cpg_solve_cases", "cpg_panel_phi_inf",
           "cpg_dub_phi_inf", "cpg_panel_v_inf", "cpg_compiled_arch", "cpg_prof_enable", "cpg_prof_read",
           "cpg_set_inf_coeff_noalloc", "cpg_measure_fp64_peak", "cpg_gemm_f32_tc", "cpg_lu_solve_f32", "cpg_release_spares", "cpg_stability_derivatives",
           "cpg_volume_velocity", "cpg_topology_wake_tris", "cpg_streamlines", "cpg_streamlines_field",
           "cpg_trefftz_wakes", "cpg_spanwise_loads",
           # cpanel_vp.h
           "cpg_ptree_build", "cpg_ptree_destroy", "cpg_ptree_info_get", "cpg_ptree_table", "cpg_ptree_host_table",
           "cpg_bh_velocity_points", "cpg_bh_particles", "cpg_ptree_set_precision", "cpg_set_particle_precision", "cpg_particles_velocity", "cpg_particles_stretch_diff",
           "cpg_panels_velocity", "cpg_panels_stretching", "cpg_vp_topology", "cpg_vpcase_create",
           "cpg_vpcase_destroy", "cpg_vpcase_info_get", "cpg_vpcase_step", "cpg_vpcase_trefftz", "cpg_vpcase_velocities", "cpg_vpcase_particles",
           "cpg_vpcase_strengths", "cpg_vpcase_surface", "cpg_vpcase_wake", "cpg_vpcase_matrices",
           # cpanel_serve.h
           "cpg_server_create", "cpg_server_destroy", "cpg_server_submit", "cpg_server_wait", "cpg_server_footprint",
           "cpg_server_submit_vp", "cpg_server_wait_vp", "cpg_server_footprint_vp",
           # cpanel_batch.h
           "cpg_group_default_shape", "cpg_set_inf_coeff_grouped", "cpg_group_schedule", "cpg_batch_solve",
           "cpg_lu_factor_grouped",
           # cpanel_io.h
           "cpg_write_cpout", "cpg_write_surface_vtu", "cpg_write_volume_vtu", "cpg_write_wake_vtu",
           "cpg_write_streamlines_vtu", "cpg_write_spanwise_csv"]

TUNE_OFF, TUNE_AUTO, TUNE_FORCE = 0, 1, 2

VEL_GAUSS_SYM, VEL_GAUSS, VEL_ALG = 1, 2, 3


class ServerParams(C.Structure):
    _fields_ = [("device", C.c_int), ("slots", C.c_int), ("budget_bytes", C.c_double), ("precision", C.c_int)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("n_body", C.c_int64), ("k", C.c_int), ("footprint_bytes", C.c_int64),
                ("queue_ms", C.c_double), ("run_ms", C.c_double), ("total_ms", C.c_double),
                ("running_at_start", C.c_int), ("message", C.c_char * 160)]


class VPResult(C.Structure):
    _fields_ = [("CL", C.c_double), ("CD", C.c_double), ("steps", C.c_int64), ("n_particles", C.c_int64),
                ("converged", C.c_int)]


class VPParams(C.Structure):
    _fields_ = [("V", C.c_double), ("alpha", C.c_double), ("beta", C.c_double), ("dt", C.c_double),
                ("cref", C.c_double), ("accelerate", C.c_int), ("Sref", C.c_double), ("mach", C.c_double),
                ("precision", C.c_int), ("run_all_steps", C.c_int)]


class VPInfo(C.Structure):
    _fields_ = [("n_body", C.c_int64), ("n_w1", C.c_int64), ("n_w2", C.c_int64), ("n_particles", C.c_int64),
                ("timestep", C.c_int64), ("solver_iters", C.c_int64), ("dt", C.c_double),
                ("n_tree_nodes", C.c_int64), ("solve_fallbacks", C.c_int64)]


class PTreeInfo(C.Structure):
    _fields_ = [("n_particles", C.c_int64), ("n_nodes", C.c_int64), ("n_leaves", C.c_int64),
                ("n_levels", C.c_int64)]


class GroupShape(C.Structure):
    _fields_ = [("chunks_per_item", C.c_int), ("near_band", C.c_int), ("blocks_per_sm", C.c_int)]


class GroupReport(C.Structure):
    _fields_ = [("shape", GroupShape), ("tuned", C.c_int), ("candidates", C.c_int), ("items", C.c_int64),
                ("pairs", C.c_int64), ("near_pairs", C.c_int64), ("ms", C.c_double)]


class BatchMesh(C.Structure):
    _fields_ = [("nodes", D), ("n_nodes", C.c_int64), ("tris", I64), ("ids", I32), ("n_tris", C.c_int64),
                ("flows", C.POINTER(Flow)), ("k", C.c_int), ("refs", Refs), ("cp", D), ("mu", D), ("CL", D),
                ("CDi", D), ("status", C.c_int), ("n_body", C.c_int64)]


class BatchParams(C.Structure):
    _fields_ = [("workers", C.c_int), ("tune", C.c_int), ("budget_bytes", C.c_double), ("lockstep", C.c_int)]


class BatchStats(C.Structure):
    _fields_ = [("ms_total", C.c_double), ("ms_topology", C.c_double), ("ms_assembly", C.c_double),
                ("ms_factor", C.c_double), ("ms_solve", C.c_double), ("waves", C.c_int), ("solves", C.c_int64), ("failed", C.c_int),
                ("group", GroupReport)]


class CpoutInputs(C.Structure):
    _fields_ = [("geom_file", C.c_char_p), ("Sref", C.c_double), ("bref", C.c_double), ("cref", C.c_double),
                ("cg", C.c_double * 3), ("velocities", D), ("n_velocities", C.c_int), ("alphas", D),
                ("n_alphas", C.c_int), ("betas", D), ("n_betas", C.c_int), ("machs", D), ("n_machs", C.c_int),
                ("subsonic_hom", C.c_int), ("surface_streamlines", C.c_int), ("stability_derivatives", C.c_int),
                ("write_inf_coeff", C.c_int), ("vortex_particles", C.c_int), ("accelerate_code", C.c_int),
                ("unsteady", C.c_int)]


class Stability(C.Structure):
    _fields_ = [("dF_dAlpha", C.c_double * 3), ("dF_dBeta", C.c_double * 3), ("dM_dAlpha", C.c_double * 3),
                ("dM_dBeta", C.c_double * 3)]


class CpoutCase(C.Structure):
    _fields_ = [("flow", Flow), ("CL", C.c_double), ("CDi", C.c_double), ("Fbody", C.c_double * 3),
                ("Fwind", C.c_double * 3), ("CM", C.c_double * 3), ("has_stability", C.c_int),
                ("stability", Stability)]


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise CpgError(7, "extension library not built: %s (run __graft_entry__.build())" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    L.cpg_create.argtypes = [C.POINTER(vp), C.c_int]
    L.cpg_destroy.argtypes = [vp]
    L.cpg_destroy.restype = None
    L.cpg_last_error.argtypes = [vp]
    L.cpg_last_error.restype = C.c_char_p
    L.cpg_set_stream.argtypes = [vp, vp]
    L.cpg_synchronize.argtypes = [vp]
    L.cpg_geometry_create.argtypes = [vp, D, C.c_int64, I64, I32, C.c_int64, C.POINTER(vp)]
    L.cpg_geometry_destroy.argtypes = [vp]
    L.cpg_geometry_destroy.restype = None
    L.cpg_geometry_info_get.argtypes = [vp, C.POINTER(GeometryInfo)]
    L.cpg_geometry_tables.argtypes = [vp, D, D, I32, D, I32]
    L.cpg_topology.argtypes = [D, C.c_int64, I64, I32, C.c_int64, C.POINTER(GeometryInfo), D, D, I32, D, I32]
    L.cpg_set_inf_coeff.argtypes = [vp, C.c_int]
    L.cpg_get_A.argtypes = [vp, D]
    L.cpg_get_B.argtypes = [vp, D]
    L.cpg_solve_cases.argtypes = [vp, C.POINTER(Flow), C.c_int, C.POINTER(Refs), C.c_int, C.POINTER(CaseOut),
                                  C.POINTER(SolveStats)]
    for f in ("cpg_panel_phi_inf",):
        getattr(L, f).argtypes = [vp, vp, vp, C.c_int64, vp, vp]
    L.cpg_dub_phi_inf.argtypes = [vp, vp, vp, C.c_int64, vp]
    L.cpg_panel_v_inf.argtypes = [vp, vp, vp, C.c_int64, vp, vp]
    L.cpg_compiled_arch.argtypes = []
    L.cpg_prof_enable.argtypes = [vp, C.c_int]
    L.cpg_prof_read.argtypes = [vp, C.POINTER(Prof)]
    L.cpg_measure_fp64_peak.argtypes = [vp, D]
    L.cpg_gemm_f32_tc.argtypes = [vp, C.c_int64, C.c_int64, C.c_int64, C.c_float, vp, C.c_int64, vp, C.c_int64,
                                  C.c_float, vp, C.c_int64, C.c_int]
    L.cpg_lu_solve_f32.argtypes = [vp, C.c_int64, vp, C.c_int64, vp]
    L.cpg_release_spares.argtypes = [vp]
    L.cpg_stability_derivatives.argtypes = [vp, C.POINTER(Flow), C.POINTER(Refs), C.c_int, C.POINTER(CaseOut),
                                            C.POINTER(Stability)]
    L.cpg_set_inf_coeff_noalloc.argtypes = [vp, C.c_int64, vp, vp, vp, C.c_int64, vp, vp, vp]
    L.cpg_ptree_build.argtypes = [vp, vp, vp, vp, C.c_int64, C.c_int64, C.c_double, C.POINTER(vp)]
    L.cpg_ptree_destroy.argtypes = [vp]
    L.cpg_ptree_destroy.restype = None
    L.cpg_ptree_info_get.argtypes = [vp, C.POINTER(PTreeInfo)]
    L.cpg_ptree_table.argtypes = [vp, D, I64]
    L.cpg_ptree_host_table.argtypes = [D, D, D, C.c_int64, C.c_int64, D, C.c_int64, I64, C.POINTER(PTreeInfo)]
    L.cpg_bh_velocity_points.argtypes = [vp, vp, C.c_int64, vp]
    L.cpg_bh_particles.argtypes = [vp, vp, vp, vp]
    L.cpg_particles_velocity.argtypes = [vp, vp, vp, vp, C.c_int64, vp, C.c_int64, C.c_int, vp]
    L.cpg_particles_stretch_diff.argtypes = [vp, vp, vp, vp, C.c_int64, vp, vp]
    L.cpg_server_create.argtypes = [C.POINTER(ServerParams), C.POINTER(vp)]
    L.cpg_server_destroy.argtypes = [vp]
    L.cpg_server_destroy.restype = None
    L.cpg_server_submit.argtypes = [vp, D, C.c_int64, I64, I32, C.c_int64, C.POINTER(Flow), C.c_int, C.POINTER(Refs),
                                    I64]
    L.cpg_server_wait.argtypes = [vp, C.c_int64, D, D, D, C.POINTER(RequestInfo)]
    L.cpg_server_footprint.argtypes = [C.c_int64, C.c_int, C.c_int]
    L.cpg_server_footprint.restype = C.c_int64
    L.cpg_server_submit_vp.argtypes = [vp, D, C.c_int64, I64, I32, C.c_int64, C.POINTER(VPParams), C.c_int,
                                       C.POINTER(C.c_int64)]
    L.cpg_server_wait_vp.argtypes = [vp, C.c_int64, C.POINTER(VPResult), D, C.POINTER(RequestInfo)]
    L.cpg_server_footprint_vp.argtypes = [C.c_int64, C.c_int64, C.c_int, C.c_int]
    L.cpg_server_footprint_vp.restype = C.c_int64
    L.cpg_panels_stretching.argtypes = [vp, vp, vp, vp, C.c_int64, vp, vp, C.c_int64, vp, vp, C.c_int64, vp]
    L.cpg_vp_topology.argtypes = [D, C.c_int64, I64, I32, C.c_int64, C.c_double, C.c_double, I64, D, D, D, I32, D, I32]
    L.cpg_vpcase_create.argtypes = [vp, D, C.c_int64, I64, I32, C.c_int64, C.POINTER(VPParams), C.POINTER(vp)]
    L.cpg_vpcase_destroy.argtypes = [vp]
    L.cpg_vpcase_destroy.restype = None
    L.cpg_vpcase_info_get.argtypes = [vp, C.POINTER(VPInfo)]
    L.cpg_ptree_set_precision.argtypes = [vp, C.c_int]
    L.cpg_set_particle_precision.argtypes = [vp, C.c_int]
    L.cpg_vpcase_step.argtypes = [vp, C.c_int]
    L.cpg_vpcase_trefftz.argtypes = [vp, D, D, C.POINTER(C.c_int)]
    L.cpg_vpcase_velocities.argtypes = [vp, C.c_int, C.c_int, D]
    L.cpg_vpcase_particles.argtypes = [vp, D, D, D, I32, I32]
    L.cpg_vpcase_strengths.argtypes = [vp, D, D, D, D]
    L.cpg_vpcase_surface.argtypes = [vp, D, C.c_double, C.c_double, D, D, D, D]
    L.cpg_vpcase_wake.argtypes = [vp, D, D]
    L.cpg_vpcase_matrices.argtypes = [vp, D, D, D]
    L.cpg_panels_velocity.argtypes = [vp, vp, vp, vp, C.c_int64, vp, vp, C.c_int64, vp, C.c_int64, vp]
    L.cpg_group_default_shape.argtypes = [C.POINTER(GroupShape)]
    L.cpg_set_inf_coeff_grouped.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.POINTER(GroupShape),
                                            C.POINTER(GroupReport)]
    L.cpg_group_schedule.argtypes = [I64, C.c_int, C.POINTER(GroupShape), I32, C.c_int64, I64, I64]
    L.cpg_batch_solve.argtypes = [vp, C.POINTER(BatchMesh), C.c_int, C.POINTER(BatchParams), C.POINTER(BatchStats)]
    L.cpg_lu_factor_grouped.argtypes = [C.POINTER(vp), C.c_int, D]
    L.cpg_write_cpout.argtypes = [C.c_char_p, C.POINTER(CpoutInputs), C.POINTER(CpoutCase), C.c_int]
    L.cpg_write_surface_vtu.argtypes = [C.c_char_p, D, C.c_int64, I64, C.c_int64, D, D, D, D, D, D, D]
    L.cpg_write_volume_vtu.argtypes = [C.c_char_p, D, C.c_int64, I64, C.c_int64, D, D]
    L.cpg_write_streamlines_vtu.argtypes = [C.c_char_p, D, D, I32, C.c_int, C.c_int]
    L.cpg_write_spanwise_csv.argtypes = [C.c_char_p, D, D, D, C.c_int]
    L.cpg_trefftz_wakes.argtypes = [vp]
    L.cpg_spanwise_loads.argtypes = [vp, C.c_int, C.c_int, D, D, D, C.POINTER(C.c_int)]
    L.cpg_volume_velocity.argtypes = [vp, D, D, D, C.c_int64, D]
    L.cpg_topology_wake_tris.argtypes = [D, C.c_int64, I64, I32, C.c_int64, I64]
    L.cpg_streamlines.argtypes = [vp, D, D, C.POINTER(Flow), D, C.c_int, C.c_double, C.c_double, C.c_int, D, D, I32,
                                  I32]
    L.cpg_streamlines_field.argtypes = [VELOCITY_FN, vp, C.c_double, D, C.c_int, C.c_double, C.c_double, C.c_int, D,
                                        D, I32, I32]
    L.cpg_write_wake_vtu.argtypes = [C.c_char_p, D, C.c_int64, I64, C.c_int64, D, D]
    _lib = L
    return L
