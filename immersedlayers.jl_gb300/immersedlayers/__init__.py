"""immersedlayers -- GB300 (sm_103a) implementation of the immersed-layer hot
path of ImmersedLayers.jl behind the same operator / cache / problem API.

All operators run as CUDA kernels in libilm.so (include/ilm.h).  Importing
this package does not require a GPU; calling an operator does, and fails
loudly when libilm.so is missing.
"""
from . import _lib
from .bodies import (Body, BodyList, circle, ellipse, from_vertices, hexagon, polygon, rectangle, square,
                     star)
from .core import (Dual, EdgeGradient, EdgeGradientPrimal, Edges, EdgesDual, EdgesPrimal, GridData, GridScaling,
                   IndexScaling, Nodes, NodesDual, NodesPrimal, PhysicalGrid, PointData, Primal, ScalarData,
                   SurfaceScalarCache, SurfaceVectorCache, TensorData, VectorData, areas, complementary_mask,
                   complementary_mask_, create_CLinvCT, create_GLinvD, create_nRTRn, create_RTLinvR, create_surface_filter,
                   create_CLinvCT_scalar, create_CL2invCT, create_GLinvD_symm, create_GLinvD_cross,
                   curl_, SurfaceFilter, ConvectiveDerivativeCache, RotConvectiveDerivativeCache,
                   convective_derivative, convective_derivative_, w_cross_v, w_cross_v_, x_gridcurl,
                   y_gridcurl, x_griddiv, y_griddiv, x_gridgrad, y_gridgrad,
                   divergence_, dot, grad_, integrate, interpolate_, inverse_laplacian_, laplacian_, mask, mask_,
                   norm, normal_cross_interpolate_, normal_dot_interpolate_, normal_interpolate_,
                   normal_interpolate_symm_, normals, ones_grid, ones_surface, points, regularize_,
                   regularize_normal_, regularize_normal_cross_, regularize_normal_dot_, regularize_normal_symm_,
                   surface_curl_, surface_curl_cross_, surface_divergence_, surface_divergence_cross_,
                   surface_divergence_symm_, surface_grad_, surface_grad_cross_, surface_grad_symm_, x_grid, y_grid,
                   zeros_grid, zeros_gridcurl, zeros_griddiv, zeros_gridgrad, zeros_surface, zeros_surfacescalar)
from .problems import (DirichletPoissonProblem, ILMProblem, ILMSystem, NeumannPoissonProblem, StokesFlowProblem,
                       construct_system, prescribed_surface_average_, prescribed_surface_jump_, solve,
                       solve_dirichlet, solve_dirichlet_refined, solve_neumann, solve_neumann_full,
                       solve_neumann_refined, solve_stokes, solve_stokes_multi, solve_stokes_multi_refined,
                       update_system_)
from .helmholtz import (ScalarPotentialCache, VectorFieldCache, VectorPotentialCache, curlv_masked_from_masked_curlv_,
                        divv_masked_from_masked_divv_, masked_curlv_from_curlv_masked_,
                        masked_divv_from_divv_masked_, scalarpotential_from_divv_, scalarpotential_from_masked_divv_,
                        scalarpotential_uniformvecfield_, vecfield_from_scalarpotential_,
                        vecfield_from_vectorpotential_, vecfield_helmholtz_, vecfield_uniformvecfield_,
                        vectorpotential_from_curlv_, vectorpotential_from_masked_curlv_,
                        vectorpotential_uniformvecfield_)
from .forcing import (AreaForcingModel, ForcingModelAndRegion, LineForcingModel, PointForcingModel, apply_forcing_,
                      forcing_regions)
from .timemarching import (ConstrainedSolution, DirichletHeatConductionProblem, HeatIntegrator, constraint, init,
                           init_sol, state, step_, temperature, timestep, timestep_fourier)

__all__ = [n for n in dir() if not n.startswith("_")]
