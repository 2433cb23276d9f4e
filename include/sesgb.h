/*
 * sesgb.h -- C ABI of the GB300 Solvent-Excluded Surface build.
 *
 * Drop-in engine for the SES build of PlathC/SESDF: the reference's C++ classes
 * bcs::Sesdf (full surface, sesdf/include/bcs/sesdf/sesdf.hpp:15-88) and
 * bcs::Ssesdf (exterior only, sesdf/include/bcs/ssesdf/ssesdf.hpp:14-77) map onto
 * the entry points below; include/bcs/ provides those classes over this ABI.
 * All pointers are plain host or device pointers, all sizes are element counts
 * unless stated otherwise, streams are passed as an opaque cudaStream_t value
 * (void*, NULL = the legacy default stream). Every entry point returns
 * SESGB_OK (0) or a negative status; sesgb_error_string() names a status and
 * sesgb_last_error() gives the message of the last failure of a context.
 */
#ifndef SESGB_H
#define SESGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SESGB_OK 0
#define SESGB_ERR_INVALID -1   /* bad argument */
#define SESGB_ERR_CUDA -2      /* a CUDA call failed */
#define SESGB_ERR_OVERFLOW -3  /* a capacity was still exceeded after regrowing */
#define SESGB_ERR_NOT_BUILT -4 /* results requested before a build */
#define SESGB_ERR_TIMEOUT -5   /* a bounded device wait gave up */
#define SESGB_ERR_MODE -6      /* request does not match the context's mode */
#define SESGB_ERR_TOO_LARGE -7 /* input beyond a fixed limit: the no-allocation sort's scratch, the cavity grid's size */

#define SESGB_MODE_FULL 0     /* bcs::Sesdf */
#define SESGB_MODE_EXTERIOR 1 /* bcs::Ssesdf */

typedef struct sesgb_ctx sesgb_ctx;

/* Build options; zero-initialise and set what you need. */
typedef struct sesgb_options
{
    uint32_t max_neighbor_per_atom; /* neighbour slots per atom, 0 = 128 (BCS_SESDF_MAXNEIGHBORPERATOM) */
    uint32_t max_intersections_per_circle; /* probes per circle used by the segment stage, 0 = 32 */
    int32_t  device;                /* CUDA device, -1 = current */
    uint32_t flags;                 /* SESGB_FLAG_* */
} sesgb_options;

/* Capture the build in a CUDA graph after its first run and replay it. */
#define SESGB_FLAG_GRAPH 1u
/* Record CUDA events between the stages of each build (see sesgb_stage_times). */
#define SESGB_FLAG_PROFILE 2u
/* Start the count-dependent output capacities at their minimum instead of at
 * protein-like multiples of the atom count: the first build then overflows, and
 * sesgb_build regrows every buffer to the counts it met (plus a quarter) and
 * builds again (sesgb_counts.rebuilds). For callers that want buffers sized to
 * their molecule rather than to the default estimate. */
#define SESGB_FLAG_MIN_CAPACITY 4u
/* Neighbour search on a grid whose cells are the largest pair cutoff (the 27
 * cells around an atom) instead of the default cells of half that cutoff (the
 * 125 cells around an atom, each row cut to the atom's reach: about half the
 * candidate pairs, for a grid eight times finer). Same neighbour lists either
 * way; for very sparse molecules, whose fine grid would be mostly empty cells. */
#define SESGB_FLAG_CUTOFF_CELLS 8u

/* Tuning knobs of a context (no counterpart in the reference): the neighbour
 * search grid and the block shapes of the three heaviest kernels. None of them
 * changes any result; sesdf_gb300/autotune.py times them on the caller's
 * molecules. Values: neighbor_cell_span 1 (cells of the largest pair cutoff) or
 * 2 (cells of half of it, the default); neighbor_warps 2, 4, 8 (default) or 16
 * warps per block of the neighbour search; visibility_warps and probe_warps 1
 * (default), 2 or 4 atoms (warps) per block of the visibility pass and the probe
 * screen; probe_queue 1 runs the probe screen as a persistent grid whose warps take
 * atoms from a work counter in sorted order (molecule by molecule, reference-grid
 * cell by cell), 0 (default) as one block per atom group. A change takes effect at
 * the next build (a captured graph is captured again). */
typedef struct sesgb_tuning
{
    uint32_t neighbor_cell_span;
    uint32_t neighbor_warps;
    uint32_t visibility_warps;
    uint32_t probe_warps;
    uint32_t probe_queue;
} sesgb_tuning;
int sesgb_set_tuning( sesgb_ctx * ctx, const sesgb_tuning * tuning );
int sesgb_get_tuning( const sesgb_ctx * ctx, sesgb_tuning * tuning );

/* Output buffers of the full-surface build: field for field the reference's
 * bcs::sesdf::SesdfData (sesdf/include/bcs/sesdf/graphics.hpp:39-66). Device pointers,
 * valid until the next build or sesgb_destroy. */
typedef struct sesgb_full_data
{
    uint32_t atomNb;
    void *   atoms; /* float4[atomNb], atoms in reference-grid order */

    uint32_t convexPatchNb;
    void *   convexPatches; /* uint2[atomNb]: [start, end) sector range per atom */

    uint32_t sectorNb;
    void *   sectors; /* float4[sectorNb]: (axis, half angle) */

    uint32_t segmentPatchNb;
    void *   segmentPatches; /* uint4[segmentPatchNb]: (i, j, probe a, probe b) */

    uint32_t circlePatchNb;
    void *   circlePatches; /* uint2[circlePatchNb]: complete circles (i, j), i < j */

    uint32_t concavePatchNb;
    void *   concavePatchesPosition;  /* float4[concavePatchNb]: (x, y, z, +-1 or +-2) */
    void *   concavePatchesId;        /* int4[concavePatchNb]: (i, j, k, neighbour count) */
    void *   concavePatchesNeighbors; /* float4[32 * singular probes] */

    float    probeRadius;
    uint16_t maxConcaveNeighbors;
} sesgb_full_data;

/* Output buffers of the exterior-only build: the reference's
 * bcs::ssesdf::SsesdfData (sesdf/include/bcs/ssesdf/graphics.hpp:29-48). */
typedef struct sesgb_exterior_data
{
    uint32_t atomNb;
    void *   atoms;

    uint32_t circlePatchNb;
    void *   circlePosition; /* float4: (torus centre, R) */
    void *   circleAxis;     /* float4: (axis, probe radius) */
    void *   circleVs;       /* float4: visibility sphere (centre - torus centre, radius) */

    uint32_t concavePatchNb;
    void *   concavePatchesPosition;
    void *   concavePatchesId;
    void *   concavePatchesNeighbors;

    float    probeRadius;
    uint16_t maxConcaveNeighbors;
} sesgb_exterior_data;

/* Counts and diagnostics of the last build. */
typedef struct sesgb_counts
{
    uint32_t atoms;
    uint32_t pairs;          /* directed circles (neighbour entries) */
    uint32_t sectors;        /* visible directed circles */
    uint32_t full_circles;   /* complete circles, i < j */
    uint32_t partial_circles;/* partial circles, i < j */
    uint32_t candidates;     /* (i, j, k) solved */
    uint32_t probes;         /* concave patches */
    uint32_t singular_probes;
    uint32_t segments;
    uint32_t tori;           /* exterior mode */
    uint32_t max_neighbors;  /* largest neighbour count seen */
    uint32_t truncated_atoms;/* atoms with more neighbours than the per-atom capacity (kept: the first ones) */
    uint32_t truncated_circles; /* circles with more probes than max_intersections_per_circle */
    uint32_t truncated_probe_neighbors; /* singular probes with more than 32 neighbours */
    uint32_t degenerate_tori; /* torus axes parallel to z (the reference produces NaN there) */
    uint32_t outside_atoms;  /* atoms outside the grid box given at creation */
    uint32_t fp64_decisions[ 7 ]; /* settled in double precision: neighbour, visibility and occlusion predicates,
                                     probe-neighbour distances, probe candidates re-solved after a float32 band hit,
                                     circles whose float32 probe order was ambiguous, kept probes whose float-float
                                     position lay too close to a float32 rounding boundary */
    uint32_t rebuilds;       /* capacity regrowths of the last build */
} sesgb_counts;

/* Reference-layout analysis buffers (sesdf/include/bcs/sesdf/sesdf.hpp:37-42). */
#define SESGB_BUF_ATOM_INDICES 0      /* uint32[atomNb]: sorted id -> input id */
#define SESGB_BUF_NEIGHBOR_COUNT 1    /* uint32[atomNb] */
#define SESGB_BUF_NEIGHBOR_IDS 2      /* uint32[atomNb * max_neighbor_per_atom] */
#define SESGB_BUF_VISIBILITY_STATUS 3 /* uint8[atomNb * max_neighbor_per_atom] (+1) */
#define SESGB_BUF_GLOBAL_TO_TRIMMED 4 /* uint32[atomNb * max_neighbor_per_atom + 1] (full mode) */

/* bcs::Sesdf::Sesdf / bcs::Ssesdf::Ssesdf (sesdf/src/sesdf/sesdf.cu:20-75,
 * sesdf/src/ssesdf/ssesdf.cu:19-66). `atoms` is a host array of n float4
 * (x, y, z, vdW radius) that stays owned by the caller and is read by every
 * sesgb_build (it may be NULL when only sesgb_build_device is used). `aabb` is
 * {min x, y, z, max x, y, z} (NULL: computed from `atoms` like getAabb,
 * sesdf/src/core/molecule.cpp:132-143). */
int sesgb_create( const float * atoms, uint32_t n, const float * aabb, float probe_radius, int mode,
                  const sesgb_options * options, sesgb_ctx ** out );

/* bcs::Sesdf::build (sesdf/src/sesdf/sesdf.cu:172-264): uploads the host atoms and
 * builds; returns when the counts are known. */
int sesgb_build( sesgb_ctx * ctx, void * stream );

/* Same build from atoms already in device memory (float4[n]). */
int sesgb_build_device( sesgb_ctx * ctx, const void * device_atoms, void * stream );

/* Asynchronous form of sesgb_build / sesgb_build_device: enqueues the whole
 * build on `stream` (device_atoms NULL = upload the borrowed host atoms) and
 * returns; sesgb_finish waits for it, and if a count exceeded a buffer's
 * capacity, regrows the buffer and builds again before returning. Results are
 * valid after sesgb_finish. */
int sesgb_build_async( sesgb_ctx * ctx, const void * device_atoms, void * stream );
int sesgb_finish( sesgb_ctx * ctx );

/* Replaces the borrowed host atom pointer (same atom count). */
int sesgb_set_host_atoms( sesgb_ctx * ctx, const float * atoms );

/* bcs::Sesdf::getData (sesdf/src/sesdf/sesdf.cu:302-344) */
int sesgb_get_full( sesgb_ctx * ctx, sesgb_full_data * out );
/* bcs::Ssesdf::getData (sesdf/src/ssesdf/ssesdf.cu:212-232) */
int sesgb_get_exterior( sesgb_ctx * ctx, sesgb_exterior_data * out );

int sesgb_get_counts( sesgb_ctx * ctx, sesgb_counts * out );

/* bcs::Sesdf::getAtomIndices (sesdf/src/sesdf/sesdf.cu:350): host copy of the
 * sorted-to-input permutation. */
int sesgb_atom_indices( sesgb_ctx * ctx, uint32_t * host_out );

/* bcs::Sesdf::getD* analysis buffers (sesdf/src/sesdf/sesdf.cu:352-356): device
 * pointer and size in bytes, in the reference's N x MaxNeighborPerAtom layout. */
int sesgb_analysis_buffer( sesgb_ctx * ctx, int which, void ** device_ptr, uint64_t * bytes );

/* Copies `bytes` from a device pointer returned by this library to host memory. */
int sesgb_copy_to_host( sesgb_ctx * ctx, const void * device_ptr, void * host, uint64_t bytes );

uint16_t sesgb_max_neighbor_per_atom( const sesgb_ctx * ctx );
uint16_t sesgb_max_intersections_per_circle( const sesgb_ctx * ctx );
uint16_t sesgb_max_intersection_neighbors( const sesgb_ctx * ctx );

/* Per-stage milliseconds of the last build (SESGB_FLAG_PROFILE): writes up to
 * `capacity` values and the number of stages; stage names by sesgb_stage_name.
 * The per-stage timers mirror app/detailed/sesdf_benchmark.inl of the reference. */
int          sesgb_stage_times( sesgb_ctx * ctx, float * ms, uint32_t capacity, uint32_t * count );
const char * sesgb_stage_name( uint32_t stage );

/* No counterpart in the reference (it allocates on every build). Sorts n atoms
 * (float4 x, y, z, vdW radius, device memory) into the order of the build's
 * `atoms` output -- the reference grid's stable cell order for `aabb` (host,
 * {min x, y, z, max x, y, z}) and `probe_radius` -- writing the sorted atoms and
 * the sorted-to-input permutation to the caller's device buffers, without
 * allocating any memory. It is for callers that cannot call cudaMalloc when
 * they need the sort: a plugin whose host application owns a fixed
 * device-memory budget and passes it every buffer, or a real-time loop that
 * must not enter the allocator (cudaMalloc may synchronise the device). Its
 * scratch is a fixed array in this library's device image (about 3.3 MB on
 * every GPU that loads the library, kept until the process exits), so n is
 * limited to SESGB_NOALLOC_MAX_ATOMS (larger n: SESGB_ERR_TOO_LARGE, nothing
 * launched). The first call on a device looks up the array's device address
 * with that device current; make that first call before any stream capture.
 * The address is kept for the life of the process: a device reset while the
 * library is loaded is not supported. All calls on a device share the array:
 * calls whose GPU work overlaps (other streams, other host threads) race on it
 * and must be serialised by the caller. A launch error left pending on the
 * calling thread by earlier work is returned as SESGB_ERR_CUDA before anything
 * is launched. */
#define SESGB_NOALLOC_MAX_ATOMS 262144u
int sesgb_sort_atoms_noalloc( const void * device_atoms, uint32_t n, const float * aabb, float probe_radius,
                              void * device_sorted_atoms, uint32_t * device_sorted_to_input, void * stream );

/* Batches (no counterpart in the reference, which builds one molecule per
 * Sesdf object): `molecules` molecules whose atoms are concatenated in `atoms`
 * (host, float4), molecule m owning atoms [molecule_start[m],
 * molecule_start[m + 1]) (molecule_start[0] = 0, non-decreasing). One build
 * covers all of them with the same fixed launch sequence as a single molecule
 * (capturable in a CUDA graph with SESGB_FLAG_GRAPH): every molecule keeps the
 * reference grid of its own construction (getAabb of its atoms), its own
 * neighbour grid and its own singular-first probe order, so that molecule m's
 * slice of the batch equals, buffer for buffer and id for id, what
 * sesgb_create + sesgb_build give for that molecule alone. The analysis buffers
 * (sesgb_analysis_buffer) stay in batch-wide numbering. */
int      sesgb_create_batch( const float * atoms, const uint32_t * molecule_start, uint32_t molecules,
                             float probe_radius, int mode, const sesgb_options * options, sesgb_ctx ** out );
uint32_t sesgb_batch_molecules( const sesgb_ctx * ctx );
/* Per-molecule record of the last build, SESGB_MOL_FIELDS values: atoms, sectors,
 * complete circles, partial circles, probes, singular probes, segments, tori, then
 * the first index of each of those in the batch buffers (atoms, sectors, complete
 * circles, partial circles, probes, singular probes, segments, tori). */
#define SESGB_MOL_FIELDS 16
int sesgb_molecule_record( const sesgb_ctx * ctx, uint32_t molecule, uint32_t * record );
/* getData of one molecule of a batch: pointers into the batch buffers, molecule-local ids. */
int sesgb_get_full_molecule( sesgb_ctx * ctx, uint32_t molecule, sesgb_full_data * out );
int sesgb_get_exterior_molecule( sesgb_ctx * ctx, uint32_t molecule, sesgb_exterior_data * out );

/* Signed distance to the SES at query points (no counterpart in the reference).
 * E = probe-centre positions outside every SAS sphere (radius r_i + rp); with
 * T = rp + SESGB_SDF_BAND: outside the SAS, sdf(x) = min_i(|x - c_i| - r_i)
 * clamped to SESGB_SDF_BAND; inside, sdf(x) = rp - min(T, dist(x, dE)), dE
 * being the SAS surface (accessible sphere patches, visible-circle arcs, probe
 * positions) of the last full-surface build. Positive outside the molecule.
 * device_queries: float3[m]; device_sdf: float[m]; device_kind (may be NULL):
 * int[m], the primitive that decided each value (0 deeper than the band, 1 atom
 * outside the SAS, 2 beyond the band outside, 3 SAS sphere, 4 circle arc, 5
 * probe). Needs a built full-surface context of one molecule. */
#define SESGB_SDF_BAND 3.0f
int sesgb_sdf( sesgb_ctx * ctx, const float * device_queries, uint32_t m, float * device_sdf, int * device_kind,
               void * stream );
/* Adjoint of sesgb_sdf: device_grad_atoms (float4[n], input atom order) receives
 * sum_q device_grad_sdf[q] * d sdf(q) / d (x, y, z, r) of every atom. The
 * primitives are searched again (nothing is kept from the forward call); a probe
 * position is differentiated by the implicit-function rule on its three
 * sphere constraints, a circle point by the Lagrange rule on its two. */
int sesgb_sdf_backward( sesgb_ctx * ctx, const float * device_queries, uint32_t m, const float * device_grad_sdf,
                        float * device_grad_atoms, void * stream );

/* Headless image of the SES of the last full-surface build of one molecule (no
 * counterpart in the reference, which draws its primitives through OpenGL): every
 * pixel's ray from a pinhole camera is sphere-traced against sesgb_sdf's signed
 * distance on the device, in one launch. Ray of pixel (ix, iy), row-major from the
 * top left: d = normalise(forward + xs right + ys up), xs = (2 (ix + 0.5) / width - 1)
 * tan_half_fov width / height, ys = (1 - 2 (iy + 0.5) / height) tan_half_fov; points
 * eye + t d from t_near. Steps never cross the surface (inside the SAS the value
 * bounds the distance to the SES, outside value - rp bounds the distance to the SAS)
 * and are at least eps / 4; a ray stops at the first point inside the SAS whose value
 * is below eps (or deeper than the band), at t_far, or after max_steps evaluations.
 * device_depth: float[width * height], t of the hit or +inf; device_normals (may be
 * NULL): float3 per pixel, the normalised central difference of the signed distance
 * (step normal_step) at the hit, 0 for a miss. Ray setup, march and normals are in
 * float32, every operation rounded on its own in the order written above. */
typedef struct sesgb_camera
{
    double   eye[ 3 ];
    double   forward[ 3 ]; /* unit vectors: view direction, image right, image up */
    double   right[ 3 ];
    double   up[ 3 ];
    double   tan_half_fov; /* tangent of half the vertical field of view */
    double   t_near, t_far;
    double   eps;          /* hit threshold, A */
    double   normal_step;  /* central-difference step of the normals, A */
    uint32_t width, height, max_steps;
} sesgb_camera;
int sesgb_render( sesgb_ctx * ctx, const sesgb_camera * camera, float * device_depth, float * device_normals,
                  void * stream );

/* Exterior and cavities (no counterpart in the reference, whose exterior-only build
 * keeps every probe, cavities included). E = probe-centre positions outside every
 * SAS sphere (radius r_i + rp) of the last build of one molecule; its component
 * that touches the border of a box around the SAS is the exterior, every other one
 * a cavity. E is sampled at voxel centres of spacing `voxel` (A, >= 0.05): origin =
 * min(c - R) - 2 voxel, dims = ceil((max(c + R) + 2 voxel - origin) / voxel) + 1 per
 * axis, at most 2^28 voxels (SESGB_ERR_TOO_LARGE otherwise), voxel (ix, iy, iz) at
 * index (ix * ny + iy) * nz + iz, accessible when ((dx^2 + dy^2) + dz^2) < R^2 holds
 * for no atom (double precision). Components are 6-connected and numbered 1..n in
 * the order of their first voxel. device_probe_component (may be NULL): int32 per
 * probe of the build, the component of the nearest accessible voxel centre among
 * the 5^3 around the probe's nearest voxel, 0 when none is accessible (E is thinner
 * than a voxel there). Synchronises `stream`; the grid stays with the context until
 * the next call. */
typedef struct sesgb_cavity_info
{
    double   origin[ 3 ]; /* centre of voxel (0, 0, 0) */
    double   voxel;
    uint32_t dims[ 3 ];
    uint32_t components; /* labels 1..components */
    uint32_t exterior;   /* components touching the grid's border */
    uint32_t cavities;   /* the others */
    uint32_t probes;     /* probes classified */
} sesgb_cavity_info;
int sesgb_cavities( sesgb_ctx * ctx, double voxel, sesgb_cavity_info * info, int32_t * device_probe_component,
                    void * stream );
/* The label grid of the last sesgb_cavities (device int32 per voxel, 0 = not accessible). */
int sesgb_cavity_labels( sesgb_ctx * ctx, const int32_t ** device_labels, uint64_t * voxels );
/* Per component k (0..components, 0 unused): voxel count and border flag (1 = exterior);
 * capacity >= components + 1. */
int sesgb_cavity_components( sesgb_ctx * ctx, uint32_t * host_voxels, uint8_t * host_border, uint32_t capacity );

/* Solvent-excluded surface area of the primitives of the last full-surface build
 * of one molecule (no counterpart in the reference): the convex patches (the
 * accessible directions of every SAS sphere, scaled to the vdW sphere), the tori
 * swept over the accessible circle arcs (trimmed at the axis where a torus
 * self-intersects) and the concave probe triangles outside the spheres of their
 * listed neighbour probes. host_parts receives double[3] = convex, toroidal,
 * concave (the total is their sum); device_atom_area (may be NULL): float[n] in
 * input order, each atom's convex patch plus half of its tori and a third of its
 * probes' concave patches. Synchronises `stream`. */
int sesgb_ses_area( sesgb_ctx * ctx, double * host_parts, float * device_atom_area, void * stream );
/* Adjoint of sesgb_ses_area: device_grad_atoms (float4[n], input atom order)
 * receives d (sum_k host_grad_parts[k] * part_k) / d (x, y, z, r) of every atom
 * (probe positions follow their atoms by the implicit-function rule). */
int sesgb_ses_area_backward( sesgb_ctx * ctx, const float * host_grad_parts, float * device_grad_atoms, void * stream );

/* Number of kernels this library has launched in this process (host-side count). */
uint64_t sesgb_launch_count( void );

/* Atoms of an MMTF structure file held in memory (data, size bytes; no compression): the first
 * model's atoms as float4 (x, y, z, vdW radius) in file order, the radius by element as the
 * reference's loader gives it (replaces bcs::load, sesdf/src/core/loader.cpp:14-71, for MMTF; the
 * C++ bcs::load of include/bcs/core/loader.hpp reads a file through it). *n receives the atom count;
 * with capacity below it nothing is written and SESGB_ERR_OVERFLOW is returned; a document that
 * cannot be read gives SESGB_ERR_INVALID. Host only, no GPU needed. */
int sesgb_load_mmtf( const void * data, size_t size, float * atoms_xyzr, uint32_t capacity, uint32_t * n );

const char * sesgb_error_string( int status );
const char * sesgb_last_error( const sesgb_ctx * ctx );
void         sesgb_destroy( sesgb_ctx * ctx );

#ifdef __cplusplus
}
#endif

#endif /* SESGB_H */
