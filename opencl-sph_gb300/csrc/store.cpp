// store.cpp -- program lists, field resolution, scratch layout and block
// maps (see store.h).
#include "store.h"

#include <stdio.h>
#include <string.h>

#include <algorithm>

namespace {

struct ProgramName {
    const char *name;
    unsigned bit;
};
// kernels/<name>.cl files of the reference (kernels/*.cl)
const ProgramName kPrograms[] = {
    {"common", PROG_COMMON},         {"fluids", PROG_FLUIDS},     {"solids", PROG_SOLIDS},
    {"solid_corotation", PROG_COROT}, {"solid_svk", PROG_SVK},     {"constraints", PROG_CONSTRAINTS},
    {"rigidbody", PROG_RIGIDBODY},
};

// Shape class of a field for the size check.
enum Shape { SCALAR, PER_PARTICLE, PER_CELL, PLANES, PER_BODY, ANY };

struct FieldReq {
    const char *name;
    char type;       // 'f' float, 'u' unsigned int
    Shape shape;
    unsigned width;  // elements per particle / scalar count / per body
};

// The fields each reference kernel file reads through USE_FIELD /
// USE_FIELD_FIRST_VALUE (kernels/common.cl, fluids.cl, solids.cl,
// solid_corotation.cl, solid_svk.cl, constraints.cl, rigidbody.cl).
const FieldReq kCommon[] = {
    {"pnum", 'u', SCALAR, 1},         {"n", 'u', SCALAR, 1},
    {"mass", 'f', SCALAR, 1},         {"timestep", 'f', SCALAR, 1},
    {"smoothingradius", 'f', SCALAR, 1}, {"gravity", 'f', SCALAR, 3},
    {"gridbounds", 'f', SCALAR, 6},   {"gridres", 'u', SCALAR, 3},
    {"position", 'f', PER_PARTICLE, 3}, {"posnext", 'f', PER_PARTICLE, 3},
    {"velocity", 'f', PER_PARTICLE, 3}, {"veleval", 'f', PER_PARTICLE, 3},
    {"acceleration", 'f', PER_PARTICLE, 3}, {"force", 'f', PER_PARTICLE, 3},
    {"density", 'f', PER_PARTICLE, 1}, {"num_neighbours", 'u', PER_PARTICLE, 1},
    {"gridcell", 'u', PER_PARTICLE, 1}, {"cellparticles", 'u', PER_PARTICLE, 1},
    {"gridcount", 'u', PER_CELL, 1},  {"celloffset", 'u', PER_CELL, 1},
    {"symmetry_planes", 'f', PLANES, 6},
    {"body_number", 'u', PER_PARTICLE, 1}, {"body_dynamic", 'u', ANY, 0},
};
const FieldReq kFluids[] = {
    {"restdens", 'f', SCALAR, 1}, {"stiffness", 'f', SCALAR, 1}, {"viscosity", 'f', SCALAR, 1},
};
const FieldReq kSolids[] = {
    {"originalpos", 'f', PER_PARTICLE, 3}, {"density0", 'f', PER_PARTICLE, 1},
};
const FieldReq kCorot[] = {
    {"rotation", 'f', PER_PARTICLE, 9},     {"strain", 'f', PER_PARTICLE, 6},
    {"stress", 'f', PER_PARTICLE, 6},       {"apq_temp", 'f', PER_PARTICLE, 9},
    {"intermediate", 'f', PER_PARTICLE, 9}, {"cutoff_force", 'f', PER_PARTICLE, 3},
    {"force_elastic", 'f', PER_PARTICLE, 3}, {"force_viscous", 'f', PER_PARTICLE, 3},
    {"padding", 'u', ANY, 0},               {"viscosity", 'f', SCALAR, 1},
    {"youngs_modulus", 'f', SCALAR, 1},     {"poisson", 'f', SCALAR, 1},
    {"originalpos", 'f', PER_PARTICLE, 3},  {"density0", 'f', PER_PARTICLE, 1},
};
const FieldReq kSvk[] = {
    {"deformation", 'f', PER_PARTICLE, 9},  {"stress", 'f', PER_PARTICLE, 6},
    {"cutoff_force", 'f', PER_PARTICLE, 3}, {"force_elastic", 'f', PER_PARTICLE, 3},
    {"force_viscous", 'f', PER_PARTICLE, 3}, {"padding", 'u', ANY, 0},
    {"viscosity", 'f', SCALAR, 1},          {"youngs_modulus", 'f', SCALAR, 1},
    {"poisson", 'f', SCALAR, 1},            {"originalpos", 'f', PER_PARTICLE, 3},
    {"density0", 'f', PER_PARTICLE, 1},
};
const FieldReq kConstraints[] = {
    {"plane_constraints", 'f', PLANES, 6}, {"plane_constraints_particles", 'u', PER_PARTICLE, 1},
};
const FieldReq kRigid[] = {
    {"body_count", 'u', SCALAR, 1},            {"body_position", 'f', PER_BODY, 3},
    {"body_euler_rotation", 'f', PER_BODY, 3}, {"rotation", 'f', PER_PARTICLE, 9},
};

template <size_t N>
bool check_all(const psdata &h, const FieldReq (&reqs)[N], unsigned pnum, unsigned cells, const char *prog,
               std::string *err) {
    for (const FieldReq &r : reqs) {
        int f = get_field_psdata(h, r.name);
        char buf[256];
        if (f < 0) {
            snprintf(buf, sizeof buf, "program '%s' needs field '%s', which the store lacks", prog, r.name);
            *err = buf;
            return false;
        }
        FieldType t = h.data_ptrs[f].type;
        if ((r.type == 'f' && t != T_FLOAT32) || (r.type == 'u' && t != T_UINT)) {
            snprintf(buf, sizeof buf, "field '%s' must be %s", r.name, r.type == 'f' ? "float" : "unsigned int");
            *err = buf;
            return false;
        }
        size_t need = 0;
        switch (r.shape) {
            case SCALAR: need = 4ull * r.width; break;
            case PER_PARTICLE: need = 4ull * r.width * pnum; break;
            case PER_CELL: need = 4ull * cells; break;
            default: need = 0;
        }
        if (h.data_sizes[f] < need) {
            snprintf(buf, sizeof buf, "field '%s' holds %u bytes, %zu needed", r.name, h.data_sizes[f], need);
            *err = buf;
            return false;
        }
    }
    return true;
}

unsigned last_dim(const psdata &h, int f) {
    unsigned nd = h.num_dimensions[f];
    return nd ? h.dimensions[h.dimensions_offsets[f] + nd - 1] : 0u;
}

template <typename T>
T *dev_field(const psdata &h, char *d_blob, const char *name) {
    int f = get_field_psdata(h, name);
    if (f < 0) return nullptr;
    return reinterpret_cast<T *>(d_blob + h.data_offsets[f]);
}

const void *host_field(const psdata &h, const char *name) {
    int f = get_field_psdata(h, name);
    return f < 0 ? nullptr : (const char *)h.data + h.data_offsets[f];
}

}  // namespace

unsigned sph_parse_programs(const char *file_list, std::string *err) {
    unsigned bits = 0;
    std::string s = file_list ? file_list : "";
    size_t i = 0;
    while (i < s.size()) {
        while (i < s.size() && strchr(", \n\r\t", s[i])) ++i;
        size_t j = i;
        while (j < s.size() && !strchr(", \n\r\t", s[j])) ++j;
        if (j > i) {
            std::string name = s.substr(i, j - i);
            bool found = false;
            for (const ProgramName &p : kPrograms)
                if (name == p.name) { bits |= p.bit; found = true; }
            if (!found) {
                *err = "unknown kernel file '" + name + "' (the reference loads kernels/<name>.cl)";
                return 0;
            }
        }
        i = j;
    }
    if (!(bits & PROG_COMMON)) {
        *err = "kernel file list must include 'common'";
        return 0;
    }
    if ((bits & PROG_COROT) && (bits & PROG_SVK)) {
        *err = "solid_corotation and solid_svk both define compute_stresses/compute_forces_solids";
        return 0;
    }
    if ((bits & (PROG_COROT | PROG_SVK)) && !(bits & PROG_SOLIDS)) {
        // the solid models build on solids.cl (density0, originalpos), as
        // every solid conf of the reference lists it
        *err = "solid_corotation and solid_svk need 'solids' in the kernel file list";
        return 0;
    }
    return bits;
}

int sph_material_of(unsigned programs) {
    if ((programs & PROG_FLUIDS) && (programs & PROG_SVK)) return MAT_MIXED;
    if (programs & PROG_COROT) return MAT_COROT;
    if (programs & PROG_SVK) return MAT_SVK;
    if (programs & PROG_FLUIDS) return MAT_FLUID;
    return -1;
}

bool sph_resolve_scene(const psdata &h, char *d, unsigned programs, SceneDesc *desc, std::string *err) {
    memset(desc, 0, sizeof(*desc));
    if (h.num_fields == 0 || !h.data) {
        *err = "empty store";
        return false;
    }
    const unsigned *pnum = (const unsigned *)host_field(h, "pnum");
    const unsigned *res = (const unsigned *)host_field(h, "gridres");
    if (!pnum || !res) {
        *err = "store lacks pnum or gridres (no neighbour grid was built)";
        return false;
    }
    unsigned long long cells = (unsigned long long)res[0] * res[1] * res[2];
    if (cells == 0 || cells > 0xFFFFFFFFull) {
        *err = "grid resolution is zero or too large";
        return false;
    }
    if (*pnum == 0) {
        *err = "pnum is zero";
        return false;
    }
    const unsigned P = *pnum, C = (unsigned)cells;
    if (!check_all(h, kCommon, P, C, "common", err)) return false;
    if ((programs & PROG_FLUIDS) && !check_all(h, kFluids, P, C, "fluids", err)) return false;
    if ((programs & PROG_SOLIDS) && !check_all(h, kSolids, P, C, "solids", err)) return false;
    if ((programs & PROG_COROT) && !check_all(h, kCorot, P, C, "solid_corotation", err)) return false;
    if ((programs & PROG_SVK) && !check_all(h, kSvk, P, C, "solid_svk", err)) return false;
    if ((programs & PROG_CONSTRAINTS) && !check_all(h, kConstraints, P, C, "constraints", err)) return false;
    if ((programs & PROG_RIGIDBODY) && !check_all(h, kRigid, P, C, "rigidbody", err)) return false;

    desc->pnum = P;
    desc->gridres[0] = res[0];
    desc->gridres[1] = res[1];
    desc->gridres[2] = res[2];
    desc->num_cells = C;
    desc->programs = programs;
    desc->jacobi_guard = 1;

    int sp = get_field_psdata(h, "symmetry_planes");
    desc->num_symmetry_planes = last_dim(h, sp);
    if (desc->num_symmetry_planes > 8 || h.data_sizes[sp] < 24u * desc->num_symmetry_planes) {
        *err = "symmetry_planes: at most 8 planes of (point, normal)";
        return false;
    }
    int pc = get_field_psdata(h, "plane_constraints");
    if (pc >= 0 && (programs & PROG_CONSTRAINTS)) {
        desc->num_plane_constraints = last_dim(h, pc);
        if (h.data_sizes[pc] < 24u * desc->num_plane_constraints) {
            *err = "plane_constraints is smaller than its last dimension says";
            return false;
        }
        if (desc->num_plane_constraints > 32) desc->num_plane_constraints = 32;
    }
    int bd = get_field_psdata(h, "body_dynamic");
    desc->body_capacity = h.data_sizes[bd] / 4u;
    if (programs & PROG_RIGIDBODY) {
        unsigned bp = h.data_sizes[get_field_psdata(h, "body_position")] / 12u;
        unsigned be = h.data_sizes[get_field_psdata(h, "body_euler_rotation")] / 12u;
        desc->body_capacity = std::min(desc->body_capacity, std::min(bp, be));
    }
    // fluids with an elastic model in one store: the extension's mixed
    // scene, whose particles carry a phase (0 fluid, 1 solid)
    if ((programs & PROG_FLUIDS) && (programs & PROG_COROT)) {
        *err = "fluids with solid_corotation in one store: the fluid-solid coupling (extension) is built for "
               "solid_svk";
        return false;
    }
    int sv = get_field_psdata(h, "solid_viscosity");
    if ((programs & PROG_FLUIDS) && (programs & PROG_SVK)) {
        const FieldReq kMixed[] = {{"phase", 'u', PER_PARTICLE, 1}};
        if (!check_all(h, kMixed, P, C, "fluids with solid_svk (mixed scene)", err)) return false;
        if (sv >= 0 && (h.data_ptrs[sv].type != T_FLOAT32 || h.data_sizes[sv] < 4u)) {
            *err = "solid_viscosity must be a float";
            return false;
        }
    }
    int wb = get_field_psdata(h, "wallbounds");
    if (wb >= 0 && (h.data_ptrs[wb].type != T_FLOAT32 || h.data_sizes[wb] < 24u)) {
        *err = "wallbounds must be 6 floats (xmin, xmax, ymin, ymax, zmin, zmax)";
        return false;
    }

    desc->n = dev_field<const unsigned>(h, d, "n");
    desc->mass = dev_field<const float>(h, d, "mass");
    desc->timestep = dev_field<const float>(h, d, "timestep");
    desc->h = dev_field<const float>(h, d, "smoothingradius");
    desc->restdens = dev_field<const float>(h, d, "restdens");
    desc->stiffness = dev_field<const float>(h, d, "stiffness");
    desc->viscosity = dev_field<const float>(h, d, "viscosity");
    desc->youngs_modulus = dev_field<const float>(h, d, "youngs_modulus");
    desc->poisson = dev_field<const float>(h, d, "poisson");
    desc->gravity = dev_field<const float>(h, d, "gravity");
    desc->gridbounds = dev_field<const float>(h, d, "gridbounds");
    desc->wallbounds = wb >= 0 ? dev_field<const float>(h, d, "wallbounds") : nullptr;
    desc->position = dev_field<float>(h, d, "position");
    desc->velocity = dev_field<float>(h, d, "velocity");
    desc->acceleration = dev_field<float>(h, d, "acceleration");
    desc->force = dev_field<float>(h, d, "force");
    desc->density = dev_field<float>(h, d, "density");
    desc->density0 = dev_field<float>(h, d, "density0");
    desc->originalpos = dev_field<float>(h, d, "originalpos");
    desc->rotation = dev_field<float>(h, d, "rotation");
    desc->strain = dev_field<float>(h, d, "strain");
    desc->stress = dev_field<float>(h, d, "stress");
    desc->apq_temp = dev_field<float>(h, d, "apq_temp");
    desc->intermediate = dev_field<float>(h, d, "intermediate");
    desc->deformation = dev_field<float>(h, d, "deformation");
    desc->cutoff_force = dev_field<float>(h, d, "cutoff_force");
    desc->force_elastic = dev_field<float>(h, d, "force_elastic");
    desc->force_viscous = dev_field<float>(h, d, "force_viscous");
    desc->num_neighbours = dev_field<unsigned>(h, d, "num_neighbours");
    desc->gridcell = dev_field<unsigned>(h, d, "gridcell");
    desc->gridcount = dev_field<unsigned>(h, d, "gridcount");
    desc->celloffset = dev_field<unsigned>(h, d, "celloffset");
    desc->cellparticles = dev_field<unsigned>(h, d, "cellparticles");
    desc->symmetry_planes = dev_field<const float>(h, d, "symmetry_planes");
    desc->plane_constraints = dev_field<const float>(h, d, "plane_constraints");
    desc->plane_constraints_particles = dev_field<const unsigned>(h, d, "plane_constraints_particles");
    desc->body_number = dev_field<const unsigned>(h, d, "body_number");
    desc->body_dynamic = dev_field<const unsigned>(h, d, "body_dynamic");
    desc->body_count = dev_field<const unsigned>(h, d, "body_count");
    desc->body_position = dev_field<float>(h, d, "body_position");
    desc->body_euler_rotation = dev_field<float>(h, d, "body_euler_rotation");
    if (programs & PROG_FLUIDS && programs & PROG_SVK) {
        desc->phase = dev_field<const unsigned>(h, d, "phase");
        desc->solid_viscosity = sv >= 0 ? dev_field<const float>(h, d, "solid_viscosity") : nullptr;
    }
    desc->num_scan_blocks = (C + SPH_SCAN_TILE - 1) / SPH_SCAN_TILE;
    return true;
}

// Rigid-body state, partial sums and per-particle offsets, for stores
// with body fields.
static size_t rigid_bytes(const SceneDesc &d) {
    if (!d.body_capacity) return 0;
    const size_t B = d.body_capacity;
    return Arena::align(8 * B * SPH_RIGID_STRIDE) + Arena::align(8 * B * SPH_RIGID_BLOCKS * SPH_RIGID_Q) +
           Arena::align(16ull * d.pnum);
}

// Sorted solid copies (rest position, stress, rotation).
static size_t solid_bytes(const SceneDesc &d) {
    if (!(d.programs & PROG_SOLIDS)) return 0;
    return Arena::align(16ull * d.pnum) + Arena::align(32ull * d.pnum) + Arena::align(48ull * d.pnum);
}

size_t sph_scratch_bytes(const SceneDesc &d) {
    size_t P = d.pnum;
    return Arena::align(4 * P)               // slot
           + Arena::align(16 * P)            // spos
           + Arena::align(16 * P)            // svel
           + Arena::align(4 * P)             // sdens
           + Arena::align(4ull * d.num_scan_blocks)
           + Arena::align(4ull * (d.num_cells + 1))
           + Arena::align(4)                 // status
           + Arena::align(4ull * SPH_MASK_WORDS * P)  // nbmask
           + Arena::align(4 * P)             // ncand
           + Arena::align(4)                 // steps_left
           + solid_bytes(d)
           + rigid_bytes(d);
}

void sph_place_scratch(SceneDesc *d, char *base) {
    size_t P = d->pnum, o = 0;
    d->slot = reinterpret_cast<unsigned *>(base + o);
    o += Arena::align(4 * P);
    d->spos = reinterpret_cast<float4 *>(base + o);
    o += Arena::align(16 * P);
    d->svel = reinterpret_cast<float4 *>(base + o);
    o += Arena::align(16 * P);
    d->sdens = reinterpret_cast<float *>(base + o);
    o += Arena::align(4 * P);
    d->scan_sums = reinterpret_cast<unsigned *>(base + o);
    o += Arena::align(4ull * d->num_scan_blocks);
    d->big_cells = reinterpret_cast<unsigned *>(base + o);
    o += Arena::align(4ull * (d->num_cells + 1));
    d->status = reinterpret_cast<unsigned *>(base + o);
    o += Arena::align(4);
    d->nbmask = reinterpret_cast<unsigned *>(base + o);
    o += Arena::align(4ull * SPH_MASK_WORDS * P);
    d->ncand = reinterpret_cast<unsigned *>(base + o);
    o += Arena::align(4 * P);
    d->steps_left = reinterpret_cast<unsigned *>(base + o);
    o += Arena::align(4);
    d->spos0 = d->sstress = d->srot = nullptr;
    if (d->programs & PROG_SOLIDS) {
        d->spos0 = reinterpret_cast<float4 *>(base + o);
        o += Arena::align(16ull * P);
        d->sstress = reinterpret_cast<float4 *>(base + o);
        o += Arena::align(32ull * P);
        d->srot = reinterpret_cast<float4 *>(base + o);
        o += Arena::align(48ull * P);
    }
    d->rigid_state = nullptr;
    d->rigid_partial = nullptr;
    d->rigid_offset = nullptr;
    if (d->body_capacity) {
        const size_t B = d->body_capacity;
        d->rigid_state = reinterpret_cast<double *>(base + o);
        o += Arena::align(8 * B * SPH_RIGID_STRIDE);
        d->rigid_partial = reinterpret_cast<double *>(base + o);
        o += Arena::align(8 * B * SPH_RIGID_BLOCKS * SPH_RIGID_Q);
        d->rigid_offset = reinterpret_cast<float4 *>(base + o);
    }
}

std::vector<unsigned> sph_rigid_bodies(const psdata &h, const SceneDesc &d) {
    std::vector<unsigned> out;
    const int f = get_field_psdata(h, "body_dynamic");
    if (f < 0 || !d.body_capacity || !d.rigid_state) return out;
    const unsigned *dyn = reinterpret_cast<const unsigned *>(static_cast<const char *>(h.data) + h.data_offsets[f]);
    unsigned count = d.body_capacity;
    const int c = get_field_psdata(h, "body_count");
    if (c >= 0) {
        const unsigned bc = *reinterpret_cast<const unsigned *>(static_cast<const char *>(h.data) + h.data_offsets[c]);
        count = std::min(count, bc);
    }
    for (unsigned b = 0; b < count; ++b)
        if (dyn[b] == SPH_BODY_RIGID) out.push_back(b + 1);
    return out;
}

void sph_build_maps(const std::vector<SceneDesc> &descs, const std::vector<unsigned> &ids, unsigned block,
                    unsigned pair_block, HostMaps *out) {
    out->particles.clear();
    out->pair_particles.clear();
    out->cells.clear();
    out->scan.clear();
    for (unsigned s : ids) {
        const SceneDesc &d = descs[s];
        for (unsigned f = 0; f < d.pnum; f += block) out->particles.push_back({s, f});
        for (unsigned f = 0; f < d.pnum; f += pair_block) out->pair_particles.push_back({s, f});
        for (unsigned f = 0; f < d.num_cells; f += block) out->cells.push_back({s, f});
        for (unsigned f = 0; f < d.num_cells; f += SPH_SCAN_TILE) out->scan.push_back({s, f});
    }
}

unsigned sph_sm_count() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 152;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) return 152;
    return (unsigned)sms;
}
