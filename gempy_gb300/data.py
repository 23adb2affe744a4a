"""Engine data types mirrored from the reference's boundary.

The reference hands these objects to ``gempy_engine.compute_model``
(``gempy/API/compute_API.py:68-73``); they are built at
``gempy/modules/data_manipulation/_engine_factory.py:14-105`` and their option
fields are serialized in ``test/test_modules/test_serialize_model.
test_generate_horizontal_stratigraphic_model.verify/Horizontal Stratigraphic
Model serialization.approved.txt:127-160``.  Only the fields the hot path
reads are mirrored, with the same names and meanings, so code written against
the engine's types works unchanged.  Coordinates are already in the engine's
transformed frame, as the reference's adapter delivers them.
"""
import enum
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

DEFAULT_SP_NUGGET = 2e-5    # gempy/core/data/surface_points.py:11
DEFAULT_ORI_NUGGET = 0.01   # gempy/core/data/orientations.py:11


class StackRelationType(enum.IntEnum):
    """Relation of a series to the older ones (``structural_frame.py:326-330``:
    the last group is always BASEMENT)."""
    ERODE = 1
    ONLAP = 2
    FAULT = 3
    BASEMENT = 4


class KernelFunction(str, enum.Enum):
    cubic = "cubic"
    exponential = "exponential"


@dataclass
class KernelOptions:
    range: float = 1.7
    c_o: float = 10.0
    uni_degree: int = 1
    i_res: float = 4.0
    gi_res: float = 2.0
    number_dimensions: int = 3
    kernel_function: KernelFunction = KernelFunction.cubic
    kernel_solver: int = 1
    compute_condition_number: bool = False
    optimizing_condition_number: bool = False
    condition_number: Optional[float] = None


@dataclass
class EvaluationOptions:
    _number_octree_levels: int = 1
    _number_octree_levels_surface: int = 4
    octree_curvature_threshold: float = -1.0
    octree_error_threshold: float = 1.0
    octree_min_level: int = 2
    mesh_extraction: bool = True
    evaluation_chunk_size: int = 500_000
    compute_scalar: bool = True
    compute_scalar_gradient: bool = False
    verbose: bool = False

    @property
    def number_octree_levels(self):
        return self._number_octree_levels

    @number_octree_levels.setter
    def number_octree_levels(self, v):
        self._number_octree_levels = int(v)

    @property
    def number_octree_levels_surface(self):
        """Levels below this one also evaluate their voxel corners (for the
        mesh extraction), and export them after the centres."""
        return self._number_octree_levels_surface

    @number_octree_levels_surface.setter
    def number_octree_levels_surface(self, v):
        self._number_octree_levels_surface = int(v)


@dataclass
class InterpolationOptions:
    kernel_options: KernelOptions = field(default_factory=KernelOptions)
    evaluation_options: EvaluationOptions = field(default_factory=EvaluationOptions)
    sigmoid_slope: float = 5_000_000
    cache_mode: int = 3
    block_solutions_type: int = 1
    debug: bool = False

    @classmethod
    def from_args(cls, range: float, c_o: float, uni_degree: int = 1, i_res: float = 4.0,
                  gi_res: float = 2.0, number_dimensions: int = 3,
                  kernel_function: KernelFunction = KernelFunction.cubic, mesh_extraction: bool = True,
                  number_octree_levels: int = 1):
        ko = KernelOptions(range=range, c_o=c_o, uni_degree=uni_degree, i_res=i_res, gi_res=gi_res,
                           number_dimensions=number_dimensions, kernel_function=kernel_function)
        eo = EvaluationOptions(_number_octree_levels=number_octree_levels, mesh_extraction=mesh_extraction)
        return cls(kernel_options=ko, evaluation_options=eo)

    @classmethod
    def init_dense_grid_options(cls):
        o = cls.from_args(range=1.7, c_o=10.0, number_octree_levels=1)
        o.block_solutions_type = 2
        return o

    @classmethod
    def init_octree_options(cls, refinement: int = 1):
        return cls.from_args(range=1.7, c_o=10.0, number_octree_levels=refinement)

    @property
    def number_octree_levels(self):
        return self.evaluation_options.number_octree_levels

    @number_octree_levels.setter
    def number_octree_levels(self, v):
        self.evaluation_options.number_octree_levels = v


@dataclass
class SurfacePoints:
    sp_coords: np.ndarray
    nugget_effect_scalar: Optional[np.ndarray] = None

    def __post_init__(self):
        self.sp_coords = np.asarray(self.sp_coords, dtype=np.float64).reshape(-1, 3)
        if self.nugget_effect_scalar is None:
            self.nugget_effect_scalar = np.full(len(self.sp_coords), DEFAULT_SP_NUGGET)
        self.nugget_effect_scalar = np.broadcast_to(
            np.asarray(self.nugget_effect_scalar, dtype=np.float64), (len(self.sp_coords),)).copy()


@dataclass
class Orientations:
    dip_positions: np.ndarray
    dip_gradients: np.ndarray
    nugget_effect_grad: Optional[np.ndarray] = None

    def __post_init__(self):
        self.dip_positions = np.asarray(self.dip_positions, dtype=np.float64).reshape(-1, 3)
        self.dip_gradients = np.asarray(self.dip_gradients, dtype=np.float64).reshape(-1, 3)
        if self.nugget_effect_grad is None:
            self.nugget_effect_grad = np.full(len(self.dip_positions), DEFAULT_ORI_NUGGET)
        self.nugget_effect_grad = np.broadcast_to(
            np.asarray(self.nugget_effect_grad, dtype=np.float64), (len(self.dip_positions),)).copy()


@dataclass
class RegularGrid:
    """Engine regular grid: cell centres of ``regular_grid_shape`` cells over
    ``orthogonal_extent`` in ``ij`` order (``regular_grid.py:58-71, 192-201``)."""
    orthogonal_extent: np.ndarray
    regular_grid_shape: np.ndarray

    def __post_init__(self):
        self.orthogonal_extent = np.asarray(self.orthogonal_extent, dtype=np.float64)
        self.regular_grid_shape = np.asarray(self.regular_grid_shape, dtype=np.int64)

    @property
    def dxdydz(self):
        e = self.orthogonal_extent
        return (e[1::2] - e[0::2]) / self.regular_grid_shape

    @property
    def origin(self):
        return self.orthogonal_extent[0::2] + self.dxdydz / 2.0

    @property
    def n_points(self):
        return int(np.prod(self.regular_grid_shape))

    @property
    def values(self):
        d = self.dxdydz
        e = self.orthogonal_extent
        axes = [np.linspace(e[2 * i] + d[i] / 2, e[2 * i + 1] - d[i] / 2, self.regular_grid_shape[i])
                for i in range(3)]
        g = np.meshgrid(*axes, indexing="ij")
        return np.stack([a.ravel() for a in g], axis=1)


@dataclass
class GenericGrid:
    values: np.ndarray

    def __post_init__(self):
        self.values = np.asarray(self.values, dtype=np.float64).reshape(-1, 3)


@dataclass
class CenteredGrid:
    """Kernel of voxels around each device, the grid behind forward gravity
    (``gp.set_centered_grid(grid, centers, resolution, radius)``,
    ``gempy/API/grid_API.py:99-108``; the engine's adapter hands it over with
    centres and radius in the transformed frame, ``gempy/modules/
    data_manipulation/_engine_factory.py:82-87``).

    Kernel per axis: x and y symmetric about the device at
    ``radius * [-g[::-1], 0, g]``, ``g = geomspace(0.01, 1, resolution // 2)``;
    z below it only, at ``-1.2 * radius * (0.05 + [0, geomspace(0.01, 1,
    resolution)])``.  With it the reference's two-layer model gives its
    gravity, -1624.1714 (``test/test_modules/test_geophysics/
    test_gravity.py:67-89``).  Each voxel reaches half-way to its neighbours and the
    outermost ones as far out as they reach in, so the voxels tile a box.
    ``kernel_grid_centers`` are relative to the device, ``left_voxel_edges`` /
    ``right_voxel_edges`` the half-widths below / above each centre (positive),
    all in ``ij`` order (x slowest); ``values`` lists every device's kernel
    points, device-major."""
    centers: np.ndarray
    resolution: np.ndarray
    radius: np.ndarray
    kernel_grid_centers: np.ndarray = field(init=False)
    left_voxel_edges: np.ndarray = field(init=False)
    right_voxel_edges: np.ndarray = field(init=False)

    def __post_init__(self):
        self.centers = np.asarray(self.centers, dtype=np.float64).reshape(-1, 3)
        self.resolution = np.asarray(self.resolution).astype(np.int64).reshape(3)
        self.radius = np.broadcast_to(np.asarray(self.radius, dtype=np.float64), (3,)).copy()
        nodes = [self._axis(int(self.resolution[a]), float(self.radius[a]), a == 2) for a in range(3)]

        def grid(k):
            m = np.meshgrid(nodes[0][k], nodes[1][k], nodes[2][k], indexing="ij")
            return np.stack([a.ravel() for a in m], axis=1)
        self.kernel_grid_centers, self.left_voxel_edges, self.right_voxel_edges = grid(0), grid(1), grid(2)

    @staticmethod
    def _axis(resolution, radius, vertical):
        if vertical:
            g = np.geomspace(0.01, 1.0, resolution)
            c = (-1.2 * radius * (0.05 + np.concatenate(([0.0], g))))[::-1]
        else:
            g = np.geomspace(0.01, 1.0, resolution // 2)
            c = radius * np.concatenate((-g[::-1], [0.0], g))
        d = np.diff(c) / 2.0
        return c, np.concatenate(([d[0]], d)), np.concatenate((d, [d[-1]]))

    @property
    def n_devices(self):
        return len(self.centers)

    @property
    def n_voxels(self):
        return len(self.kernel_grid_centers)

    @property
    def values(self):
        return (self.centers[:, None, :] + self.kernel_grid_centers[None]).reshape(-1, 3)


@dataclass
class GeophysicsInput:
    """``tz`` per kernel voxel (``calculate_gravity_gradient``) and the
    density of every lithology id (1-based), as the reference's
    ``GeophysicsInput(tz, densities)`` (``test_gravity.py:74-78``)."""
    tz: np.ndarray
    densities: np.ndarray


@dataclass
class EngineGrid:
    octree_grid: Optional[RegularGrid] = None
    dense_grid: Optional[RegularGrid] = None
    topography: Optional[GenericGrid] = None
    sections: Optional[GenericGrid] = None
    custom_grid: Optional[GenericGrid] = None
    geophysics_grid: Optional[object] = None


@dataclass
class InterpolationInput:
    surface_points: SurfacePoints
    orientations: Orientations
    grid: EngineGrid
    unit_values: np.ndarray
    weights: list = field(default_factory=list)


@dataclass
class TensorsStructure:
    number_of_points_per_surface: np.ndarray

    def __post_init__(self):
        self.number_of_points_per_surface = np.asarray(self.number_of_points_per_surface, dtype=np.int64)


@dataclass
class StacksStructure:
    """Per-stack sizes and relations.  ``faults_relations[j, i]`` true: the
    FAULT stack j offsets the younger stack i (``structural_frame.py:244-273``)."""
    number_of_points_per_stack: np.ndarray
    number_of_orientations_per_stack: np.ndarray
    number_of_surfaces_per_stack: np.ndarray
    masking_descriptor: List[StackRelationType]
    faults_relations: Optional[np.ndarray] = None

    def __post_init__(self):
        self.number_of_points_per_stack = np.asarray(self.number_of_points_per_stack, dtype=np.int64)
        self.number_of_orientations_per_stack = np.asarray(self.number_of_orientations_per_stack, dtype=np.int64)
        self.number_of_surfaces_per_stack = np.asarray(self.number_of_surfaces_per_stack, dtype=np.int64)
        self.masking_descriptor = [StackRelationType(int(r)) for r in self.masking_descriptor]
        n = len(self.number_of_points_per_stack)
        if self.faults_relations is not None:
            fr = np.asarray(self.faults_relations, dtype=bool)
            if fr.shape != (n, n):
                raise ValueError(f"faults_relations must be {n} x {n}")
            for j, i in zip(*np.nonzero(fr)):
                if j >= i:
                    raise ValueError(f"stack {j} cannot offset the older or same stack {i}")
                if self.masking_descriptor[j] != StackRelationType.FAULT:
                    raise ValueError(f"stack {j} offsets stack {i} but is not a FAULT stack")
            self.faults_relations = fr

    @property
    def n_stacks(self):
        return len(self.number_of_points_per_stack)

    def fault_sources(self, i):
        """The FAULT stacks that offset stack i, oldest first."""
        if self.faults_relations is None:
            return []
        return [int(j) for j in np.nonzero(self.faults_relations[:, i])[0]]


@dataclass
class InputDataDescriptor:
    """Per-series partition of the inputs (``structural_frame.py:306-317``)."""
    tensors_structure: TensorsStructure
    stack_structure: StacksStructure

    @classmethod
    def from_arrays(cls, points_per_surface, surfaces_per_stack, orientations_per_stack, relations,
                    faults_relations=None):
        pps = np.asarray(points_per_surface, dtype=np.int64)
        sps = np.asarray(surfaces_per_stack, dtype=np.int64)
        bounds = np.concatenate([[0], np.cumsum(sps)])
        pts = np.array([pps[bounds[i]:bounds[i + 1]].sum() for i in range(len(sps))], dtype=np.int64)
        rel = list(relations)
        rel[-1] = StackRelationType.BASEMENT
        return cls(TensorsStructure(pps), StacksStructure(pts, orientations_per_stack, sps, rel, faults_relations))

    @classmethod
    def from_structural_frame(cls, structural_frame, making_descriptor=None, faults_relations=None,
                              faults_input_data=None):
        """The descriptor the reference builds from a ``StructuralFrame``
        (``gempy/core/data/structural_frame.py:306-317``): one stack per
        structural group, surfaces per group, surface points per element,
        orientations per group, the groups' relations (the last one BASEMENT)
        and the fault relations.  ``structural_frame`` needs the attributes the
        reference's frame has: ``structural_groups``, each with ``elements``
        (each with ``number_of_points`` and ``number_of_orientations``) and
        ``structural_relation``.  ``faults_input_data`` (finite-fault
        thickness/offset) is accepted and must be unset: this path models
        infinite faults."""
        if faults_input_data is not None and any(f is not None for f in faults_input_data):
            raise NotImplementedError("finite faults (faults_input_data) are not part of this path")
        groups = list(structural_frame.structural_groups)
        pps, sps, ops, rels = [], [], [], []
        for g in groups:
            els = list(g.elements)
            sps.append(len(els))
            pps.extend(int(e.number_of_points) for e in els)
            ops.append(int(sum(int(e.number_of_orientations) for e in els)))
            rels.append(_relation(g.structural_relation))
        if making_descriptor is not None:
            rels = [_relation(r) for r in making_descriptor]
        if faults_relations is None:
            faults_relations = getattr(structural_frame, "fault_relations", None)
        return cls.from_arrays(pps, sps, ops, rels, faults_relations)


def _relation(r):
    """StackRelationType from an enum of this module, the reference's own enum
    (matched by name) or an int."""
    if isinstance(r, StackRelationType):
        return r
    name = getattr(r, "name", None)
    if name is not None and name in StackRelationType.__members__:
        return StackRelationType[name]
    return StackRelationType(int(r))


# ----------------------------------------------------------------------------- outputs


@dataclass
class ExportedFields:
    scalar_field: np.ndarray
    gx_field: Optional[np.ndarray] = None
    gy_field: Optional[np.ndarray] = None
    gz_field: Optional[np.ndarray] = None
    scalar_field_at_surface_points: Optional[np.ndarray] = None


@dataclass
class InterpOutput:
    """Per-series output at one point set."""
    exported_fields: ExportedFields
    values_block: np.ndarray
    weights: Optional[np.ndarray] = None
    mask: Optional[np.ndarray] = None

    @property
    def scalar_field(self):
        return self.exported_fields.scalar_field

    @property
    def ids_block(self):
        return np.rint(self.values_block).astype(np.int32)


@dataclass
class CombinedOutput:
    exported_fields: ExportedFields
    block: np.ndarray
    ids_block: np.ndarray
    mask_matrix: Optional[np.ndarray] = None


@dataclass
class OctreeLevel:
    """One octree level.  ``outputs`` holds one evaluation per series over
    the level's grid: the voxel centres, followed by the 8 corners of every
    voxel (corner order x slowest, z fastest) on levels below
    ``number_octree_levels_surface``, where the corners are evaluated for the
    mesh extraction.  ``last_output_center`` is the combined block at the
    centres, ``last_output_corners`` at the corners (or None)."""
    grid_centers: np.ndarray
    dxdydz: np.ndarray
    outputs_centers: List[InterpOutput]
    last_output_center: CombinedOutput
    last_output_corners: Optional[CombinedOutput] = None
    grid_corners: Optional[np.ndarray] = None

    @property
    def outputs(self):
        return self.outputs_centers


@dataclass
class RootOutput:
    outputs: List[InterpOutput]


@dataclass
class RawArraysSolution:
    lith_block: Optional[np.ndarray] = None
    scalar_field_matrix: Optional[np.ndarray] = None
    mask_matrix_squeezed: Optional[np.ndarray] = None
    custom: Optional[np.ndarray] = None
    block_matrix: Optional[np.ndarray] = None


@dataclass
class Solutions:
    octrees_output: List[OctreeLevel]
    root_output: RootOutput
    raw_arrays: RawArraysSolution
    scalar_field_at_surface_points: List[float]
    _ordered_elements: List[np.ndarray]
    block_solution_type: int = 1
    dc_meshes: Optional[list] = None
    gravity: Optional[np.ndarray] = None
    timings: dict = field(default_factory=dict)
    solver_info: list = field(default_factory=list)
    taped_interpolation_input: Optional[object] = None   # leaf tensors of a compute_grads run
