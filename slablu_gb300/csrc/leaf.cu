// Leaf kernels: launchers, FP64 residual, solution assembly, and the
// standalone batched leaf DtN entry point.
#include "leaf.cuh"

namespace slab {

template <typename T, bool kMixed>
static int leaf_factor_launch(cudaStream_t s, const LeafFactorArgs<T>& a, int nleaf, int ctas_per_sm) {
  const size_t bytes = leaf_smem_for_occupancy(reinterpret_cast<const void*>(leaf_factor_kernel<T, kMixed>),
                                               leaf_factor_smem_bytes(a.p, sizeof(T)), ctas_per_sm);
  SLAB_TRY(ensure_smem(leaf_factor_kernel<T, kMixed>, bytes, "leaf_factor"));
  leaf_factor_kernel<T, kMixed><<<nleaf, kNT, bytes, s>>>(a);
  SLAB_CHECK_LAUNCH();
  return SLAB_OK;
}

template <typename T>
int leaf_factor(cudaStream_t s, const LeafFactorArgs<T>& a, int nleaf, int ctas_per_sm) {
  if (nleaf <= 0) return SLAB_OK;
  if (a.preassembled && a.nxa == 0) {
    const size_t bytes = 7 * (size_t)a.p * a.p * sizeof(double) + 2 * (size_t)a.n;
    SLAB_TRY(ensure_smem(leaf_assemble_kernel<T>, bytes, "leaf_assemble"));
    leaf_assemble_kernel<T><<<nleaf, kNT, bytes, s>>>(a);
    SLAB_CHECK_LAUNCH();
  }
  if (a.nx > 2 * kCT || a.nxa > 2 * kCT) return set_error(SLAB_ERR_ARG, "leaf_factor: p = %d too large", a.p);
  if (a.nxa > 0) {  // mixed derivative: Jxreorder columns and the interpolation stage
    if (!a.co.c12 || !a.interp || !a.jxr)
      return set_error(SLAB_ERR_ARG, "leaf_factor: c12, interp and jxreorder are needed together");
    // the interpolation stage holds Interp_mat and 32 rows of X in the dynamic shared memory
    if (((size_t)a.nxa * a.nx + 32 * (size_t)a.nxa) * sizeof(T) > leaf_factor_smem_bytes(a.p, sizeof(T)))
      return set_error(SLAB_ERR_ARG, "leaf_factor: p = %d too small for the interpolation stage", a.p);
    return leaf_factor_launch<T, true>(s, a, nleaf, ctas_per_sm);
  }
  return leaf_factor_launch<T, false>(s, a, nleaf, ctas_per_sm);
}

size_t leaf_smem_for_occupancy(const void* kernel, size_t need, int ctas_per_sm) {
  if (ctas_per_sm <= 0) return need;
  int dev = 0, per_sm = 0, reserved = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess) {
    cudaGetLastError();
    return need;
  }
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) {
    cudaGetLastError();
    return need;
  }
  // the largest dynamic size with which at most ctas_per_sm blocks fit one SM
  const long long cap = (long long)per_sm / ctas_per_sm - reserved - (long long)fa.sharedSizeBytes;
  const long long b = cap / 128 * 128;
  return b > (long long)need ? (size_t)b : need;
}

template int leaf_factor<float>(cudaStream_t, const LeafFactorArgs<float>&, int, int);
template int leaf_factor<double>(cudaStream_t, const LeafFactorArgs<double>&, int, int);

__global__ void __launch_bounds__(256) residual_kernel(ResidualArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int p = a.p, q = a.q, n = a.n, nx = a.nx;
  double* Dsh = reinterpret_cast<double*>(smem_raw);
  double* Dsqsh = Dsh + p * p;
  double* u = Dsqsh + p * p;
  const int leaf = blockIdx.x;
  const int tid = threadIdx.x;
  for (int i = tid; i < p * p; i += blockDim.x) {
    Dsh[i] = a.D[i];
    Dsqsh[i] = a.Dsq[i];
  }
  const int lofs = leaf * p * p;
  const LeafCoeffs& co = a.co;
  for (int c = 0; c < a.nrhs; ++c) {
    __syncthreads();
    for (int i = tid; i < p * p; i += blockDim.x) u[i] = 0.0;
    __syncthreads();
    for (int r = tid; r < n; r += blockDim.x) {
      int i1, i2;
      interior_node(r, q, i1, i2);
      u[i1 * p + i2] = a.uc[((size_t)leaf * a.nrhs + c) * n + r];
    }
    for (int s = tid; s < nx; s += blockDim.x) {
      int j1, j2;
      face_node(s, p, q, j1, j2);
      u[j1 * p + j2] = a.ux[a.leafglob[(size_t)leaf * nx + s] + (size_t)c * a.ntot];
    }
    __syncthreads();
    for (int r = tid; r < n; r += blockDim.x) {
      int i1, i2;
      interior_node(r, q, i1, i2);
      const int k = lofs + i1 * p + i2;
      double t11 = 0, t22 = 0, t1 = 0, t2 = 0;
      if (co.c1 || co.c2) {
        for (int j = 0; j < p; ++j) {
          const double ux1 = u[j * p + i2], ux2 = u[i1 * p + j];
          t11 += Dsqsh[i1 * p + j] * ux1;
          t22 += Dsqsh[i2 * p + j] * ux2;
          t1 += Dsh[i1 * p + j] * ux1;
          t2 += Dsh[i2 * p + j] * ux2;
        }
      } else {
        // no first-order terms: half the FP64 products (this kernel is FP64-pipe bound)
        for (int j = 0; j < p; ++j) {
          t11 += Dsqsh[i1 * p + j] * u[j * p + i2];
          t22 += Dsqsh[i2 * p + j] * u[i1 * p + j];
        }
      }
      double Au = 0.0;
      if (co.c11) Au -= co.c11[k] * t11;
      if (co.c22) Au -= co.c22[k] * t22;
      if (co.c1) Au -= co.c1[k] * t1;
      if (co.c2) Au -= co.c2[k] * t2;
      if (co.c) Au += co.c[k] * u[i1 * p + i2];
      const double f = a.fbody ? a.fbody[(size_t)k + (size_t)c * a.nleaf * p * p] : 0.0;
      a.rc[((size_t)leaf * a.nrhs + c) * n + r] = f - Au;
    }
    for (int s = tid; s < nx; s += blockDim.x) {
      const int g = a.leafglob[(size_t)leaf * nx + s];
      if (a.dirmask[g]) continue;
      const int f = s / q, t = s % q + 1;
      double flux = 0.0;
      // Nx rows: [-D1[Jl]; D1[Jr]; -D2[Jd]; D2[Ju]] with D1 = -kron(D,I), D2 = -kron(I,D)
      if (f == 0)
        for (int j = 0; j < p; ++j) flux += Dsh[j] * u[j * p + t];
      else if (f == 1)
        for (int j = 0; j < p; ++j) flux -= Dsh[(p - 1) * p + j] * u[j * p + t];
      else if (f == 2)
        for (int j = 0; j < p; ++j) flux += Dsh[j] * u[t * p + j];
      else
        for (int j = 0; j < p; ++j) flux -= Dsh[(p - 1) * p + j] * u[t * p + j];
      atomicAdd(&a.rx[g + (size_t)c * a.ntot], -flux);
    }
  }
}

__global__ void __launch_bounds__(256) residual_mixed_kernel(ResidualArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int p = a.p, q = a.q, n = a.n, nx = a.nx, nxa = a.nxa, pp = p * p;
  double* Dsh = reinterpret_cast<double*>(smem_raw);
  double* Dsqsh = Dsh + pp;
  double* u = Dsqsh + pp;  // leaf node values
  double* W = u + pp;      // U D^T
  double* uf = W + pp;     // the leaf's nx face values
  const int leaf = blockIdx.x;
  const int tid = threadIdx.x;
  for (int i = tid; i < pp; i += blockDim.x) {
    Dsh[i] = a.D[i];
    Dsqsh[i] = a.Dsq[i];
  }
  const int lofs = leaf * pp;
  const LeafCoeffs& co = a.co;
  for (int c = 0; c < a.nrhs; ++c) {
    __syncthreads();
    for (int i = tid; i < pp; i += blockDim.x) u[i] = 0.0;
    for (int s = tid; s < nx; s += blockDim.x) uf[s] = a.ux[a.leafglob[(size_t)leaf * nx + s] + (size_t)c * a.ntot];
    __syncthreads();
    for (int r = tid; r < n; r += blockDim.x) {
      int i1, i2;
      interior_node(r, q, i1, i2);
      u[i1 * p + i2] = a.uc[((size_t)leaf * a.nrhs + c) * n + r];
    }
    // the interpolated boundary (faces and corners), Interp_mat u_faces
    for (int t = tid; t < nxa; t += blockDim.x) {
      double v = 0.0;
      for (int s = 0; s < nx; ++s) v += a.interp[(size_t)t * nx + s] * uf[s];
      u[a.jxr[t]] = v;
    }
    __syncthreads();
    for (int idx = tid; idx < pp; idx += blockDim.x) {
      const int j1 = idx / p, i2 = idx % p;
      double w = 0.0;
      for (int j2 = 0; j2 < p; ++j2) w += u[j1 * p + j2] * Dsh[i2 * p + j2];
      W[idx] = w;
    }
    __syncthreads();
    for (int r = tid; r < n; r += blockDim.x) {
      int i1, i2;
      interior_node(r, q, i1, i2);
      const int k = lofs + i1 * p + i2;
      double t11 = 0, t22 = 0, t1 = 0, t2 = 0, t12 = 0;
      for (int j = 0; j < p; ++j) {
        const double ux1 = u[j * p + i2], ux2 = u[i1 * p + j];
        t11 += Dsqsh[i1 * p + j] * ux1;
        t22 += Dsqsh[i2 * p + j] * ux2;
        t1 += Dsh[i1 * p + j] * ux1;
        t2 += Dsh[i2 * p + j] * ux2;
        t12 += Dsh[i1 * p + j] * W[j * p + i2];
      }
      double Au = 0.0;
      if (co.c11) Au -= co.c11[k] * t11;
      if (co.c22) Au -= co.c22[k] * t22;
      if (co.c12) Au += (-2.0 * co.c12[k]) * t12;
      if (co.c1) Au -= co.c1[k] * t1;
      if (co.c2) Au -= co.c2[k] * t2;
      if (co.c) Au += co.c[k] * u[i1 * p + i2];
      const double f = a.fbody ? a.fbody[(size_t)k + (size_t)c * a.nleaf * p * p] : 0.0;
      a.rc[((size_t)leaf * a.nrhs + c) * n + r] = f - Au;
    }
    __syncthreads();
    // the flux rows see the face values themselves (Nx has no corner columns)
    for (int s = tid; s < nx; s += blockDim.x) {
      int j1, j2;
      face_node(s, p, q, j1, j2);
      u[j1 * p + j2] = uf[s];
    }
    __syncthreads();
    for (int s = tid; s < nx; s += blockDim.x) {
      const int g = a.leafglob[(size_t)leaf * nx + s];
      if (a.dirmask[g]) continue;
      const int f = s / q, t = s % q + 1;
      double flux = 0.0;
      if (f == 0)
        for (int j = 0; j < p; ++j) flux += Dsh[j] * u[j * p + t];
      else if (f == 1)
        for (int j = 0; j < p; ++j) flux -= Dsh[(p - 1) * p + j] * u[j * p + t];
      else if (f == 2)
        for (int j = 0; j < p; ++j) flux += Dsh[j] * u[t * p + j];
      else
        for (int j = 0; j < p; ++j) flux -= Dsh[(p - 1) * p + j] * u[t * p + j];
      atomicAdd(&a.rx[g + (size_t)c * a.ntot], -flux);
    }
  }
}

__global__ void __launch_bounds__(256) residual_t_kernel(ResidualArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int p = a.p, q = a.q, n = a.n, nx = a.nx;
  double* Dsh = reinterpret_cast<double*>(smem_raw);
  double* Dsqsh = Dsh + p * p;
  double* m11 = Dsqsh + p * p;  // -c11 lam, -c22 lam, -c1 lam, -c2 lam on the p x p grid
  double* m22 = m11 + p * p;
  double* m1 = m22 + p * p;
  double* m2 = m1 + p * p;
  double* lx = m2 + p * p;      // lambda on the leaf's face nodes (0 on Dirichlet faces)
  const int leaf = blockIdx.x;
  const int tid = threadIdx.x;
  for (int i = tid; i < p * p; i += blockDim.x) {
    Dsh[i] = a.D[i];
    Dsqsh[i] = a.Dsq[i];
  }
  const int lofs = leaf * p * p;
  const LeafCoeffs& co = a.co;
  for (int c = 0; c < a.nrhs; ++c) {
    __syncthreads();
    for (int i = tid; i < p * p; i += blockDim.x) m11[i] = m22[i] = m1[i] = m2[i] = 0.0;
    __syncthreads();
    for (int r = tid; r < n; r += blockDim.x) {
      int i1, i2;
      interior_node(r, q, i1, i2);
      const int k = i1 * p + i2;
      const double l = a.uc[((size_t)leaf * a.nrhs + c) * n + r];
      if (co.c11) m11[k] = -co.c11[lofs + k] * l;
      if (co.c22) m22[k] = -co.c22[lofs + k] * l;
      if (co.c1) m1[k] = -co.c1[lofs + k] * l;
      if (co.c2) m2[k] = -co.c2[lofs + k] * l;
    }
    for (int s = tid; s < nx; s += blockDim.x) {
      const int g = a.leafglob[(size_t)leaf * nx + s];
      lx[s] = a.dirmask[g] ? 0.0 : a.ux[g + (size_t)c * a.ntot];
    }
    __syncthreads();
    // z[l] = sum_k Aloc[k,l] lam_k + sum_s Nx[s,l] lx_s at interior and face nodes l
    for (int idx = tid; idx < n + nx; idx += blockDim.x) {
      int l1, l2;
      if (idx < n)
        interior_node(idx, q, l1, l2);
      else
        face_node(idx - n, p, q, l1, l2);
      const int l = l1 * p + l2;
      double z = 0.0;
      if (co.c1 || co.c2) {
        for (int k1 = 0; k1 < p; ++k1) {
          z += Dsqsh[k1 * p + l1] * m11[k1 * p + l2];
          z += Dsh[k1 * p + l1] * m1[k1 * p + l2];
        }
        for (int k2 = 0; k2 < p; ++k2) {
          z += Dsqsh[k2 * p + l2] * m22[l1 * p + k2];
          z += Dsh[k2 * p + l2] * m2[l1 * p + k2];
        }
      } else {  // no first-order terms: their (zero) products skipped
        for (int k1 = 0; k1 < p; ++k1) z += Dsqsh[k1 * p + l1] * m11[k1 * p + l2];
        for (int k2 = 0; k2 < p; ++k2) z += Dsqsh[k2 * p + l2] * m22[l1 * p + k2];
      }
      if (idx < n && co.c) z += co.c[lofs + l] * a.uc[((size_t)leaf * a.nrhs + c) * n + idx];
      // Nx^T lx: face rows couple the nodes on their normal line
      if (l2 >= 1 && l2 <= p - 2) {
        const int sL = l2 - 1, sR = q + l2 - 1;
        z += Dsh[l1] * lx[sL];                  // left face row (0, l2): D[0, l1]
        z -= Dsh[(p - 1) * p + l1] * lx[sR];    // right face row (p-1, l2): -D[p-1, l1]
      }
      if (l1 >= 1 && l1 <= p - 2) {
        const int sD = 2 * q + l1 - 1, sU = 3 * q + l1 - 1;
        z += Dsh[l2] * lx[sD];                  // down face row (l1, 0): D[0, l2]
        z -= Dsh[(p - 1) * p + l2] * lx[sU];    // up face row (l1, p-1): -D[p-1, l2]
      }
      if (idx < n) {
        const double g = a.fbody ? a.fbody[((size_t)leaf * a.nrhs + c) * n + idx] : 0.0;
        a.rc[((size_t)leaf * a.nrhs + c) * n + idx] = g - z;
      } else {
        const int gf = a.leafglob[(size_t)leaf * nx + (idx - n)];
        if (a.all_faces || !a.dirmask[gf]) atomicAdd(&a.rx[gf + (size_t)c * a.ntot], -z);
      }
    }
  }
}

// Transposed residual with a mixed derivative: the PDE rows see every leaf node
// (the boundary through Interp_mat, corners included), so their part of
// A^T lam is formed on the whole p x p grid and carried back to the face
// columns by Interp_mat^T; the flux rows see the interior and face nodes only.
__global__ void __launch_bounds__(256) residual_t_mixed_kernel(ResidualArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int p = a.p, q = a.q, n = a.n, nx = a.nx, nxa = a.nxa, pp = p * p;
  double* Dsh = reinterpret_cast<double*>(smem_raw);
  double* Dsqsh = Dsh + pp;
  double* m11 = Dsqsh + pp;  // -c11 lam, -c22 lam, -2 c12 lam, -c1 lam, -c2 lam on the grid
  double* m22 = m11 + pp;
  double* m12 = m22 + pp;
  double* m1 = m12 + pp;
  double* m2 = m1 + pp;
  double* V = m2 + pp;       // m12 D
  double* zp = V + pp;       // PDE-row part of A^T lam at every leaf node
  double* lx = zp + pp;      // lambda on the leaf's face nodes (0 on Dirichlet faces)
  const int leaf = blockIdx.x;
  const int tid = threadIdx.x;
  for (int i = tid; i < pp; i += blockDim.x) {
    Dsh[i] = a.D[i];
    Dsqsh[i] = a.Dsq[i];
  }
  const int lofs = leaf * pp;
  const LeafCoeffs& co = a.co;
  for (int c = 0; c < a.nrhs; ++c) {
    __syncthreads();
    for (int i = tid; i < pp; i += blockDim.x) m11[i] = m22[i] = m12[i] = m1[i] = m2[i] = 0.0;
    __syncthreads();
    for (int r = tid; r < n; r += blockDim.x) {
      int i1, i2;
      interior_node(r, q, i1, i2);
      const int k = i1 * p + i2;
      const double l = a.uc[((size_t)leaf * a.nrhs + c) * n + r];
      if (co.c11) m11[k] = -co.c11[lofs + k] * l;
      if (co.c22) m22[k] = -co.c22[lofs + k] * l;
      if (co.c12) m12[k] = (-2.0 * co.c12[lofs + k]) * l;
      if (co.c1) m1[k] = -co.c1[lofs + k] * l;
      if (co.c2) m2[k] = -co.c2[lofs + k] * l;
    }
    for (int s = tid; s < nx; s += blockDim.x) {
      const int g = a.leafglob[(size_t)leaf * nx + s];
      lx[s] = a.dirmask[g] ? 0.0 : a.ux[g + (size_t)c * a.ntot];
    }
    __syncthreads();
    for (int idx = tid; idx < pp; idx += blockDim.x) {
      const int k1 = idx / p, l2 = idx % p;
      double v = 0.0;
      for (int k2 = 0; k2 < p; ++k2) v += m12[k1 * p + k2] * Dsh[k2 * p + l2];
      V[idx] = v;
    }
    __syncthreads();
    // zp[l] = sum_k Aloc[k, l] lam_k over the interior rows k, at every node l
    for (int idx = tid; idx < pp; idx += blockDim.x) {
      const int l1 = idx / p, l2 = idx % p;
      double z = 0.0;
      for (int k1 = 0; k1 < p; ++k1) {
        z += Dsqsh[k1 * p + l1] * m11[k1 * p + l2];
        z += Dsh[k1 * p + l1] * m1[k1 * p + l2];
        z += Dsh[k1 * p + l1] * V[k1 * p + l2];
      }
      for (int k2 = 0; k2 < p; ++k2) {
        z += Dsqsh[k2 * p + l2] * m22[l1 * p + k2];
        z += Dsh[k2 * p + l2] * m2[l1 * p + k2];
      }
      zp[idx] = z;
    }
    __syncthreads();
    for (int idx = tid; idx < n + nx; idx += blockDim.x) {
      int l1, l2;
      if (idx < n)
        interior_node(idx, q, l1, l2);
      else
        face_node(idx - n, p, q, l1, l2);
      const int l = l1 * p + l2;
      // Nx^T lx: face rows couple the nodes on their normal line (never a corner)
      double z = 0.0;
      if (l2 >= 1 && l2 <= p - 2) {
        z += Dsh[l1] * lx[l2 - 1];
        z -= Dsh[(p - 1) * p + l1] * lx[q + l2 - 1];
      }
      if (l1 >= 1 && l1 <= p - 2) {
        z += Dsh[l2] * lx[2 * q + l1 - 1];
        z -= Dsh[(p - 1) * p + l2] * lx[3 * q + l1 - 1];
      }
      if (idx < n) {
        z += zp[l];
        if (co.c) z += co.c[lofs + l] * a.uc[((size_t)leaf * a.nrhs + c) * n + idx];
        const double g = a.fbody ? a.fbody[((size_t)leaf * a.nrhs + c) * n + idx] : 0.0;
        a.rc[((size_t)leaf * a.nrhs + c) * n + idx] = g - z;
      } else {
        const int s = idx - n;
        for (int t = 0; t < nxa; ++t) z += a.interp[(size_t)t * nx + s] * zp[a.jxr[t]];
        const int gf = a.leafglob[(size_t)leaf * nx + s];
        if (a.all_faces || !a.dirmask[gf]) atomicAdd(&a.rx[gf + (size_t)c * a.ntot], -z);
      }
    }
  }
}

__global__ void __launch_bounds__(256) assemble_t_kernel(AssembleTArgs a) {
  const int p = a.p, q = a.q, n = a.n, nx = a.nx;
  const int leaf = blockIdx.x, tid = threadIdx.x;
  const int nr = 4 * (p - 1);
  const size_t ldo = (size_t)a.nleaf * p * p;
  for (int c = 0; c < a.nrhs; ++c) {
    const double* ds = a.dsol + (size_t)leaf * p * p + c * ldo;
    for (int r = tid; r < n; r += blockDim.x) {
      int i1, i2;
      interior_node(r, q, i1, i2);
      a.gint[((size_t)leaf * a.nrhs + c) * n + r] = ds[i1 * p + i2];
    }
    for (int s = tid; s < nx; s += blockDim.x) {
      const int g = a.leafglob[(size_t)leaf * nx + s];
      double v = 0.0;
      for (int t = 0; t < nr; ++t) v += a.interp[(size_t)t * nx + s] * ds[a.jxreorder[t]];
      atomicAdd(&a.gfaces[g + (size_t)c * a.ntot], v);
    }
  }
}

__global__ void __launch_bounds__(256) coeff_grad_kernel(GradArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int p = a.p, q = a.q, n = a.n, nx = a.nx;
  double* Dsh = reinterpret_cast<double*>(smem_raw);
  double* Dsqsh = Dsh + p * p;
  double* u = Dsqsh + p * p;
  const int leaf = blockIdx.x, tid = threadIdx.x;
  for (int i = tid; i < p * p; i += blockDim.x) {
    Dsh[i] = a.D[i];
    Dsqsh[i] = a.Dsq[i];
  }
  const int lofs = leaf * p * p;
  const size_t ldl = (size_t)a.nleaf * p * p;
  // boundary nodes of the leaf carry no PDE row: zero gradient there
  for (int i = tid; i < p * p; i += blockDim.x) {
    const int i1 = i / p, i2 = i % p;
    if (i1 == 0 || i1 == p - 1 || i2 == 0 || i2 == p - 1) {
      if (a.g0) a.g0[lofs + i] = 0.0;
      if (a.g11) a.g11[lofs + i] = 0.0;
      if (a.g22) a.g22[lofs + i] = 0.0;
      if (a.g1) a.g1[lofs + i] = 0.0;
      if (a.g2) a.g2[lofs + i] = 0.0;
    }
  }
  // each interior node is owned by one thread across all right-hand sides
  constexpr int kMaxOwn = 4;  // n <= kMaxOwn * blockDim.x (p <= 33 at 256 threads)
  double acc[kMaxOwn][5];
#pragma unroll
  for (int o = 0; o < kMaxOwn; ++o)
#pragma unroll
    for (int t = 0; t < 5; ++t) acc[o][t] = 0.0;
  for (int c = 0; c < a.nrhs; ++c) {
    __syncthreads();
    for (int i = tid; i < p * p; i += blockDim.x) u[i] = 0.0;
    __syncthreads();
    for (int r = tid; r < n; r += blockDim.x) {
      int i1, i2;
      interior_node(r, q, i1, i2);
      u[i1 * p + i2] = a.uleaf[lofs + i1 * p + i2 + c * ldl];
    }
    for (int s = tid; s < nx; s += blockDim.x) {
      int j1, j2;
      face_node(s, p, q, j1, j2);
      u[j1 * p + j2] = a.ufaces[a.leafglob[(size_t)leaf * nx + s] + (size_t)c * a.ntot];
    }
    __syncthreads();
#pragma unroll
    for (int o = 0; o < kMaxOwn; ++o) {
      const int r = tid + o * blockDim.x;
      if (r >= n) break;
      int i1, i2;
      interior_node(r, q, i1, i2);
      const int k = i1 * p + i2;
      const double l = a.lam[lofs + k + c * ldl];
      double t11 = 0, t22 = 0, t1 = 0, t2 = 0;
      for (int j = 0; j < p; ++j) {
        const double ux1 = u[j * p + i2], ux2 = u[i1 * p + j];
        t11 += Dsqsh[i1 * p + j] * ux1;
        t22 += Dsqsh[i2 * p + j] * ux2;
        t1 += Dsh[i1 * p + j] * ux1;
        t2 += Dsh[i2 * p + j] * ux2;
      }
      acc[o][0] += l * t11;
      acc[o][1] += l * t22;
      acc[o][2] += l * t1;
      acc[o][3] += l * t2;
      acc[o][4] -= l * u[k];
    }
  }
#pragma unroll
  for (int o = 0; o < kMaxOwn; ++o) {
    const int r = tid + o * blockDim.x;
    if (r >= n) break;
    int i1, i2;
    interior_node(r, q, i1, i2);
    const int k = lofs + i1 * p + i2;
    if (a.g11) a.g11[k] = acc[o][0];
    if (a.g22) a.g22[k] = acc[o][1];
    if (a.g1) a.g1[k] = acc[o][2];
    if (a.g2) a.g2[k] = acc[o][3];
    if (a.g0) a.g0[k] = acc[o][4];
  }
}

// Coefficient gradients with a mixed derivative: the PDE rows see the
// interpolated boundary u[Jxreorder] = Interp_mat u_faces (corners included),
// and dL/dc12_k = 2 lam_k (D12 u)_k with D12 u = D U D^T on the leaf grid.
__global__ void __launch_bounds__(256) coeff_grad_mixed_kernel(GradArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int p = a.p, q = a.q, n = a.n, nx = a.nx, nxa = a.nxa, pp = p * p;
  double* Dsh = reinterpret_cast<double*>(smem_raw);
  double* Dsqsh = Dsh + pp;
  double* u = Dsqsh + pp;
  double* W = u + pp;   // U D^T
  double* uf = W + pp;  // the leaf's nx face values
  const int leaf = blockIdx.x, tid = threadIdx.x;
  for (int i = tid; i < pp; i += blockDim.x) {
    Dsh[i] = a.D[i];
    Dsqsh[i] = a.Dsq[i];
  }
  const int lofs = leaf * pp;
  const size_t ldl = (size_t)a.nleaf * pp;
  double* outs[6] = {a.g11, a.g22, a.g1, a.g2, a.g0, a.g12};
  for (int i = tid; i < pp; i += blockDim.x) {
    const int i1 = i / p, i2 = i % p;
    if (i1 == 0 || i1 == p - 1 || i2 == 0 || i2 == p - 1)
      for (int t = 0; t < 6; ++t)
        if (outs[t]) outs[t][lofs + i] = 0.0;
  }
  constexpr int kMaxOwn = 4;  // n <= kMaxOwn * blockDim.x
  double acc[kMaxOwn][6];
#pragma unroll
  for (int o = 0; o < kMaxOwn; ++o)
#pragma unroll
    for (int t = 0; t < 6; ++t) acc[o][t] = 0.0;
  for (int c = 0; c < a.nrhs; ++c) {
    __syncthreads();
    for (int i = tid; i < pp; i += blockDim.x) u[i] = 0.0;
    for (int s = tid; s < nx; s += blockDim.x) uf[s] = a.ufaces[a.leafglob[(size_t)leaf * nx + s] + (size_t)c * a.ntot];
    __syncthreads();
    for (int r = tid; r < n; r += blockDim.x) {
      int i1, i2;
      interior_node(r, q, i1, i2);
      u[i1 * p + i2] = a.uleaf[lofs + i1 * p + i2 + c * ldl];
    }
    for (int t = tid; t < nxa; t += blockDim.x) {
      double v = 0.0;
      for (int s = 0; s < nx; ++s) v += a.interp[(size_t)t * nx + s] * uf[s];
      u[a.jxr[t]] = v;
    }
    __syncthreads();
    for (int idx = tid; idx < pp; idx += blockDim.x) {
      const int j1 = idx / p, i2 = idx % p;
      double w = 0.0;
      for (int j2 = 0; j2 < p; ++j2) w += u[j1 * p + j2] * Dsh[i2 * p + j2];
      W[idx] = w;
    }
    __syncthreads();
#pragma unroll
    for (int o = 0; o < kMaxOwn; ++o) {
      const int r = tid + o * blockDim.x;
      if (r >= n) break;
      int i1, i2;
      interior_node(r, q, i1, i2);
      const int k = i1 * p + i2;
      const double l = a.lam[lofs + k + c * ldl];
      double t11 = 0, t22 = 0, t1 = 0, t2 = 0, t12 = 0;
      for (int j = 0; j < p; ++j) {
        const double ux1 = u[j * p + i2], ux2 = u[i1 * p + j];
        t11 += Dsqsh[i1 * p + j] * ux1;
        t22 += Dsqsh[i2 * p + j] * ux2;
        t1 += Dsh[i1 * p + j] * ux1;
        t2 += Dsh[i2 * p + j] * ux2;
        t12 += Dsh[i1 * p + j] * W[j * p + i2];
      }
      acc[o][0] += l * t11;
      acc[o][1] += l * t22;
      acc[o][2] += l * t1;
      acc[o][3] += l * t2;
      acc[o][4] -= l * u[k];
      acc[o][5] += 2.0 * l * t12;
    }
  }
#pragma unroll
  for (int o = 0; o < kMaxOwn; ++o) {
    const int r = tid + o * blockDim.x;
    if (r >= n) break;
    int i1, i2;
    interior_node(r, q, i1, i2);
    const int k = lofs + i1 * p + i2;
    for (int t = 0; t < 6; ++t)
      if (outs[t]) outs[t][k] = acc[o][t];
  }
}

// Leaf-node solution: interior values copied, boundary nodes (faces and corners)
// through Interp_mat from the face values, kAssembleRhs right-hand sides per
// pass.  Each row of Interp_mat is summed over its nonzero span only (one face's
// nodes), in the same column order as the dense sum.
__global__ void __launch_bounds__(256) assemble_solution_kernel(AssembleArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* uxl = reinterpret_cast<double*>(smem_raw);  // nx x kAssembleRhs
  const int p = a.p, q = a.q, n = a.n, nx = a.nx;
  const int leaf = blockIdx.x, tid = threadIdx.x;
  const int nr = 4 * (p - 1);
  const size_t ldo = (size_t)a.nleaf * p * p;
  for (int c0 = 0; c0 < a.nrhs; c0 += kAssembleRhs) {
    const int gc = min(kAssembleRhs, a.nrhs - c0);
    __syncthreads();
    for (int idx = tid; idx < nx * gc; idx += blockDim.x) {
      const int s = idx % nx, c = idx / nx;
      uxl[s + c * nx] = a.ux[a.leafglob[(size_t)leaf * nx + s] + (size_t)(c0 + c) * a.ntot];
    }
    __syncthreads();
    for (int idx = tid; idx < nr * gc; idx += blockDim.x) {
      const int t = idx % nr, c = idx / nr;
      const int lo = a.ispan ? a.ispan[2 * t] : 0, hi = a.ispan ? a.ispan[2 * t + 1] : nx;
      double v = 0.0;
      for (int s = lo; s < hi; ++s) v += a.interp[(size_t)t * nx + s] * uxl[s + c * nx];
      a.out[(size_t)leaf * p * p + (c0 + c) * ldo + a.jxreorder[t]] = v;
    }
    for (int idx = tid; idx < n * gc; idx += blockDim.x) {
      const int r = idx % n, c = idx / n;
      int i1, i2;
      interior_node(r, q, i1, i2);
      a.out[(size_t)leaf * p * p + (c0 + c) * ldo + i1 * p + i2] = a.uc[((size_t)leaf * a.nrhs + c0 + c) * n + r];
    }
  }
}

namespace {

__global__ void transpose_out_kernel(const float* in, double* out, int nx, int nleaf) {
  const long long tot = (long long)nleaf * nx * nx;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const long long l = i / ((long long)nx * nx);
    const int rem = (int)(i % ((long long)nx * nx));
    const int r = rem / nx, c = rem % nx;  // out row-major (r, c)
    out[i] = (double)in[l * nx * nx + r + (long long)c * nx];
  }
}
__global__ void transpose_out_kernel(const double* in, double* out, int nx, int nleaf) {
  const long long tot = (long long)nleaf * nx * nx;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const long long l = i / ((long long)nx * nx);
    const int rem = (int)(i % ((long long)nx * nx));
    const int r = rem / nx, c = rem % nx;
    out[i] = in[l * nx * nx + r + (long long)c * nx];
  }
}

// S (column-major n x nx inside G) -> row-major n x nx doubles
template <typename T>
__global__ void copy_S_kernel(const T* G, long long strideG, int n, int nx, int nleaf, double* S) {
  const long long tot = (long long)nleaf * n * nx;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const long long l = i / ((long long)n * nx);
    const int rem = (int)(i % ((long long)n * nx));
    const int r = rem / nx, c = rem % nx;
    S[i] = (double)G[l * strideG + (long long)n * n + r + (long long)c * n];
  }
}

// nxa: extra columns of the leaf system (4(p-2) face nodes; 4(p-1) Jxreorder
// nodes with a mixed derivative, plus room for the interpolation matrix).
template <typename T>
size_t leaf_work_bytes(int nleaf, int p, bool mixed = false) {
  const int q = p - 2, n = q * q, nx = 4 * q, nxa = mixed ? 4 * (p - 1) : nx;
  size_t b = 0;
  auto add = [&](size_t bytes) { b += (bytes + 255) / 256 * 256; };
  add((size_t)nleaf * n * (n + nxa) * sizeof(T));  // G
  add((size_t)nleaf * n * sizeof(int));            // pivots
  add((size_t)nleaf * nx * nx * sizeof(T));        // DtN (T)
  add((size_t)nx * n * sizeof(T));                 // Nxc
  add((size_t)nx * nx * sizeof(T));                // Nxx
  if (mixed) add((size_t)nxa * nx * sizeof(T));    // interpolation matrix
  return b;
}

template <typename T>
__global__ void to_type_kernel(const double* in, T* out, int count) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) out[i] = (T)in[i];
}

template <typename T>
int leaf_dtn_impl(int nleaf, int p, const LeafCoeffs& co, const double* D, const double* Dsq, const double* Nx,
                  void* work, size_t work_bytes, double* dtn_out, double* S_out, int* info, cudaStream_t s,
                  const double* interp = nullptr, const int* jxr = nullptr) {
  const int q = p - 2, n = q * q, nx = 4 * q;
  const bool mixed = co.c12 != nullptr;
  const int nxa = mixed ? 4 * (p - 1) : nx;
  if (mixed && (!interp || !jxr)) return set_error(SLAB_ERR_ARG, "slab_leaf_dtn_mixed: interp and jxreorder needed");
  if (mixed && ((size_t)nxa * nx + 32 * (size_t)nxa) * sizeof(T) > leaf_factor_smem_bytes(p, sizeof(T)))
    return set_error(SLAB_ERR_ARG, "slab_leaf_dtn_mixed: p = %d too small for the interpolation stage", p);
  if (work_bytes < leaf_work_bytes<T>(nleaf, p, mixed)) return set_error(SLAB_ERR_ARG, "slab_leaf_dtn: work too small");
  unsigned char* w = static_cast<unsigned char*>(work);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    void* ptr = w + off;
    off += (bytes + 255) / 256 * 256;
    return ptr;
  };
  T* G = static_cast<T*>(take((size_t)nleaf * n * (n + nxa) * sizeof(T)));
  int* piv = static_cast<int*>(take((size_t)nleaf * n * sizeof(int)));
  T* dtn = static_cast<T*>(take((size_t)nleaf * nx * nx * sizeof(T)));
  T* Nxc = static_cast<T*>(take((size_t)nx * n * sizeof(T)));
  T* Nxx = static_cast<T*>(take((size_t)nx * nx * sizeof(T)));
  split_nx_kernel<T><<<64, 256, 0, s>>>(Nx, p, q, Nxc, Nxx);
  SLAB_CHECK_LAUNCH();
  LeafFactorArgs<T> a{};
  a.p = p; a.q = q; a.n = n; a.nx = nx;
  a.co = co; a.D = D; a.Dsq = Dsq; a.Nxc = Nxc; a.Nxx = Nxx;
  a.G = G; a.strideG = (long long)n * (n + nxa); a.piv = piv; a.dtn = dtn; a.info = info;
  a.decouple = 0;
  a.preassembled = 0;
  if (mixed) {
    T* interpT = static_cast<T*>(take((size_t)nxa * nx * sizeof(T)));
    to_type_kernel<T><<<ceil_div(nxa * nx, 256), 256, 0, s>>>(interp, interpT, nxa * nx);
    SLAB_CHECK_LAUNCH();
    a.nxa = nxa;
    a.interp = interpT;
    a.jxr = jxr;
  }
  SLAB_TRY(leaf_factor<T>(s, a, nleaf));
  transpose_out_kernel<<<1024, 256, 0, s>>>(dtn, dtn_out, nx, nleaf);
  SLAB_CHECK_LAUNCH();
  if (S_out) {
    copy_S_kernel<T><<<1024, 256, 0, s>>>(G, a.strideG, n, nx, nleaf, S_out);
    SLAB_CHECK_LAUNCH();
  }
  return SLAB_OK;
}

}  // namespace

// Leaf DtN maps with a caller-provided work area (no allocation).
int leaf_dtn_with_work(int nleaf, int p, const LeafCoeffs& co, const double* D, const double* Dsq, const double* Nx,
                       int precision, void* work, size_t work_bytes, double* dtn_out, double* S_out, int* info,
                       cudaStream_t s) {
  if (precision == SLAB_PREC_FP64)
    return leaf_dtn_impl<double>(nleaf, p, co, D, Dsq, Nx, work, work_bytes, dtn_out, S_out, info, s);
  return leaf_dtn_impl<float>(nleaf, p, co, D, Dsq, Nx, work, work_bytes, dtn_out, S_out, info, s);
}

}  // namespace slab

extern "C" size_t slab_leaf_dtn_work_bytes(int nleaf, int p, int precision) {
  if (nleaf <= 0 || p < 4) return 0;
  return precision == SLAB_PREC_FP64 ? slab::leaf_work_bytes<double>(nleaf, p)
                                     : slab::leaf_work_bytes<float>(nleaf, p);
}

extern "C" size_t slab_leaf_dtn_mixed_work_bytes(int nleaf, int p, int precision) {
  if (nleaf <= 0 || p < 4) return 0;
  return precision == SLAB_PREC_FP64 ? slab::leaf_work_bytes<double>(nleaf, p, true)
                                     : slab::leaf_work_bytes<float>(nleaf, p, true);
}

extern "C" int slab_leaf_dtn_mixed(int nleaf, int p, const double* c11, const double* c22, const double* c12,
                                   const double* c1, const double* c2, const double* c, const double* D,
                                   const double* Dsq, const double* Nx, const double* interp, const int* jxreorder,
                                   int precision, void* work, size_t work_bytes, double* dtn, double* S, int* info,
                                   void* stream) {
  if (nleaf <= 0 || p < 4 || !D || !Dsq || !Nx || !interp || !jxreorder || !work || !dtn)
    return slab::set_error(SLAB_ERR_ARG, "slab_leaf_dtn_mixed: invalid argument");
  if (precision != SLAB_PREC_FP64 && precision != SLAB_PREC_FP32 && precision != SLAB_PREC_MIXED)
    return slab::set_error(SLAB_ERR_ARG, "slab_leaf_dtn_mixed: unknown precision %d", precision);
  slab::LeafCoeffs co{c11, c22, c1, c2, c, c12};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!c12)  // no mixed derivative: the face-node system of slab_leaf_dtn
    return precision == SLAB_PREC_FP64
               ? slab::leaf_dtn_impl<double>(nleaf, p, co, D, Dsq, Nx, work, work_bytes, dtn, S, info, s)
               : slab::leaf_dtn_impl<float>(nleaf, p, co, D, Dsq, Nx, work, work_bytes, dtn, S, info, s);
  if (precision == SLAB_PREC_FP64)
    return slab::leaf_dtn_impl<double>(nleaf, p, co, D, Dsq, Nx, work, work_bytes, dtn, S, info, s, interp,
                                       jxreorder);
  return slab::leaf_dtn_impl<float>(nleaf, p, co, D, Dsq, Nx, work, work_bytes, dtn, S, info, s, interp, jxreorder);
}

extern "C" int slab_leaf_dtn(int nleaf, int p, const double* c11, const double* c22, const double* c1,
                             const double* c2, const double* c, const double* D, const double* Dsq,
                             const double* Nx, int precision, void* work, size_t work_bytes, double* dtn,
                             double* S, int* info, void* stream) {
  if (nleaf <= 0 || p < 4 || !D || !Dsq || !Nx || !work || !dtn)
    return slab::set_error(SLAB_ERR_ARG, "slab_leaf_dtn: invalid argument");
  if (precision != SLAB_PREC_FP64 && precision != SLAB_PREC_FP32 && precision != SLAB_PREC_MIXED)
    return slab::set_error(SLAB_ERR_ARG, "slab_leaf_dtn: unknown precision %d", precision);
  slab::LeafCoeffs co{c11, c22, c1, c2, c};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (precision == SLAB_PREC_FP64)
    return slab::leaf_dtn_impl<double>(nleaf, p, co, D, Dsq, Nx, work, work_bytes, dtn, S, info, s);
  return slab::leaf_dtn_impl<float>(nleaf, p, co, D, Dsq, Nx, work, work_bytes, dtn, S, info, s);
}
