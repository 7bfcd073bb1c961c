/* C entry points over the reference's own code compiled for the host
 * (oracle/build_ref.sh, Thrust OpenMP backend).  They call the reference's
 * functions exactly as its Python binding does (src/isoext_ext.cu:95-109,
 * 329-378) and copy the results into malloc'd host arrays.
 * TEST INFRASTRUCTURE ONLY: used to pin the oracle and make golden fixtures. */
#include "dc.cuh"
#include "grid/sparse.cuh"
#include "grid/uniform.cuh"
#include "its.cuh"
#include "mc/mc.cuh"

#include <cstdlib>
#include <cstring>
#include <string>

namespace {
thread_local std::string g_err;

template <typename T> T *dup(const T *src, size_t n) {
    T *p = (T *)malloc((n ? n : 1) * sizeof(T));
    if (n) memcpy(p, src, n * sizeof(T));
    return p;
}

void out_mesh(NDArray<float3> &v, NDArray<int> &f, float **vo, long long *nv, int **fo,
              long long *nf) {
    *nv = (long long)v.size();
    *nf = (long long)(f.size() / 3);
    *vo = dup((const float *)v.data(), v.size() * 3);
    *fo = dup(f.data(), f.size());
}

std::unique_ptr<Grid> dense(const float *vals, int nx, int ny, int nz, const float *amin,
                            const float *amax) {
    auto g = std::make_unique<UniformGrid>(make_uint3(nx, ny, nz),
                                           make_float3(amin[0], amin[1], amin[2]),
                                           make_float3(amax[0], amax[1], amax[2]));
    NDArray<float> in(const_cast<float *>(vals), {(size_t)nx, (size_t)ny, (size_t)nz});
    g->set_values(in);
    return g;
}

std::unique_ptr<SparseGrid> sparse(const int *ids, const float *vals, long long n, int nx, int ny,
                                   int nz, const float *amin, const float *amax) {
    auto g = std::make_unique<SparseGrid>(make_uint3(nx, ny, nz),
                                          make_float3(amin[0], amin[1], amin[2]),
                                          make_float3(amax[0], amax[1], amax[2]));
    NDArray<uint> idn(reinterpret_cast<uint *>(const_cast<int *>(ids)), {(size_t)n});
    g->add_cells(idn);
    NDArray<float> in(const_cast<float *>(vals), {(size_t)n, 8});
    g->set_values(in);
    return g;
}
}  // namespace

extern "C" {

const char *ref_last_error() { return g_err.c_str(); }
void ref_free(void *p) { free(p); }

int ref_mc_dense(const float *vals, int nx, int ny, int nz, const float *amin, const float *amax,
                 float level, const char *method, float **v, long long *nv, int **f,
                 long long *nf) {
    try {
        auto g = dense(vals, nx, ny, nz, amin, amax);
        auto [V, F] = mc::marching_cubes(g.get(), level, method);
        out_mesh(V, F, v, nv, f, nf);
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}

int ref_mc_sparse(const int *ids, const float *vals, long long n, int nx, int ny, int nz,
                  const float *amin, const float *amax, float level, const char *method,
                  float **v, long long *nv, int **f, long long *nf) {
    try {
        auto g = sparse(ids, vals, n, nx, ny, nz, amin, amax);
        auto [V, F] = mc::marching_cubes(g.get(), level, method);
        out_mesh(V, F, v, nv, f, nf);
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}

/* Intersection of a dense grid.  Arrays are malloc'd; ncross = K, nactive = A. */
int ref_intersection_dense(const float *vals, int nx, int ny, int nz, const float *amin,
                           const float *amax, float level, int normals, float **pts,
                           float **nrm, unsigned **edges, unsigned char **is_out,
                           unsigned **cells, unsigned **offsets, long long *ncross,
                           long long *nactive) {
    try {
        auto g = dense(vals, nx, ny, nz, amin, amax);
        Intersection its = get_intersection(g.get(), level, normals != 0);
        *ncross = (long long)its.points.size();
        *nactive = (long long)its.cell_indices.size();
        *pts = dup((const float *)its.points.data(), its.points.size() * 3);
        *nrm = dup((const float *)its.normals.data(), its.normals.size() * 3);
        *edges = dup((const unsigned *)its.edges.data(), its.edges.size() * 2);
        *is_out = (unsigned char *)malloc(its.is_out.size() ? its.is_out.size() : 1);
        for (size_t i = 0; i < its.is_out.size(); i++) (*is_out)[i] = its.is_out.data()[i];
        *cells = dup(its.cell_indices.data(), its.cell_indices.size());
        *offsets = dup(its.cell_offsets.data(), its.cell_offsets.size());
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}

/* Dual contouring of a dense grid.  normals == NULL: automatic normals (the
 * binding's default path); otherwise user normals [K,3] set on the
 * intersection, as isoext.dual_contouring(grid, intersection=its) does. */
int ref_dc_dense(const float *vals, int nx, int ny, int nz, const float *amin, const float *amax,
                 float level, const float *normals, long long nnormals, float reg, float svd_tol,
                 float **v, long long *nv, int **f, long long *nf) {
    try {
        auto g = dense(vals, nx, ny, nz, amin, amax);
        Intersection its = get_intersection(g.get(), level, normals == nullptr);
        if (normals) {
            if ((long long)its.points.size() != nnormals)
                throw std::runtime_error("normal count does not match the intersections");
            NDArray<float3> nn(reinterpret_cast<float3 *>(const_cast<float *>(normals)),
                               {(size_t)nnormals});
            its.set_normals(nn);
        }
        auto [V, F] = dual_contouring(g.get(), its, level, reg, svd_tol);
        out_mesh(V, F, v, nv, f, nf);
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}

int ref_dc_sparse(const int *ids, const float *vals, long long n, int nx, int ny, int nz,
                  const float *amin, const float *amax, float level, float reg, float svd_tol,
                  float **v, long long *nv, int **f, long long *nf) {
    try {
        auto g = sparse(ids, vals, n, nx, ny, nz, amin, amax);
        Intersection its = get_intersection(g.get(), level, true);
        auto [V, F] = dual_contouring(g.get(), its, level, reg, svd_tol);
        out_mesh(V, F, v, nv, f, nf);
        return 0;
    } catch (const std::exception &e) {
        g_err = e.what();
        return -1;
    }
}

}  // extern "C"
