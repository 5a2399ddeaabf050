// Builds pRRTC's Environment<float> (src/collision/environment.hh) on the
// device from flat float arrays, for the harnesses in this directory (test
// infrastructure; included after the reference headers).
//
// pRRTC builds its Environment<float> on the host and byte-copies the
// obstacle structs to the device (pRRTC.cu:130-222).  Here the same structs
// are filled in device code, so the host never needs the structs' layout
// (their Shape base holds a std::string whose bytes the checker never reads;
// no constructor runs, exactly as with the byte copy).
//
// Flat layouts (floats per obstacle): sphere 4 (x y z r); capsule 8
// (x1 y1 z1 xv yv zv r rdv); cuboid 15 (x y z, axis1 xyz, axis2 xyz, axis3
// xyz, r1 r2 r3).  Cylinders are never read by the reference checker
// (utils.cuh:211-242) and are not taken.
#pragma once

// Bytes of scratch the host must provide for an environment with the given
// counts: every struct rounded up to 16 bytes, plus the Environment itself.
extern "C" __global__ void ref_env_bytes(unsigned long long *out)
{
    out[0] = sizeof(Environment<float>);
    out[1] = sizeof(Sphere<float>);
    out[2] = sizeof(Capsule<float>);
    out[3] = sizeof(Cuboid<float>);
    out[4] = alignof(Environment<float>);
}

template <class T>
__device__ T *carve(unsigned char *&p, int n)
{
    T *r = reinterpret_cast<T *>(p);
    p += ((sizeof(T) * (size_t)n + 255) / 256) * 256;
    return n ? r : nullptr;
}

// One thread: lays out Environment<float> and its arrays in `scratch`
// (256-byte aligned, at least the size ref_env_bytes implies).
extern "C" __global__ void ref_env_build(unsigned char *scratch, const float *sph, int ns, const float *cap, int nc,
                                         const float *zcap, int nzc, const float *cub, int ncb, const float *zcub,
                                         int nzb)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned char *p = scratch;
    Environment<float> *env = carve<Environment<float>>(p, 1);
    Sphere<float> *s = carve<Sphere<float>>(p, ns);
    Capsule<float> *c = carve<Capsule<float>>(p, nc);
    Capsule<float> *zc = carve<Capsule<float>>(p, nzc);
    Cuboid<float> *b = carve<Cuboid<float>>(p, ncb);
    Cuboid<float> *zb = carve<Cuboid<float>>(p, nzb);
    for (int i = 0; i < ns; i++) {
        const float *f = sph + 4 * i;
        s[i].x = f[0]; s[i].y = f[1]; s[i].z = f[2]; s[i].r = f[3];
        s[i].min_distance = 0.0f;
    }
    auto caps = [](Capsule<float> *d, const float *src, int n) {
        for (int i = 0; i < n; i++) {
            const float *f = src + 8 * i;
            d[i].x1 = f[0]; d[i].y1 = f[1]; d[i].z1 = f[2];
            d[i].xv = f[3]; d[i].yv = f[4]; d[i].zv = f[5];
            d[i].r = f[6]; d[i].rdv = f[7];
            d[i].min_distance = 0.0f;
        }
    };
    caps(c, cap, nc);
    caps(zc, zcap, nzc);
    auto cubs = [](Cuboid<float> *d, const float *src, int n) {
        for (int i = 0; i < n; i++) {
            const float *f = src + 15 * i;
            d[i].x = f[0]; d[i].y = f[1]; d[i].z = f[2];
            d[i].axis_1_x = f[3]; d[i].axis_1_y = f[4]; d[i].axis_1_z = f[5];
            d[i].axis_2_x = f[6]; d[i].axis_2_y = f[7]; d[i].axis_2_z = f[8];
            d[i].axis_3_x = f[9]; d[i].axis_3_y = f[10]; d[i].axis_3_z = f[11];
            d[i].axis_1_r = f[12]; d[i].axis_2_r = f[13]; d[i].axis_3_r = f[14];
            d[i].min_distance = 0.0f;
        }
    };
    cubs(b, cub, ncb);
    cubs(zb, zcub, nzb);
    env->spheres = s;
    env->num_spheres = (unsigned)ns;
    env->capsules = c;
    env->num_capsules = (unsigned)nc;
    env->z_aligned_capsules = zc;
    env->num_z_aligned_capsules = (unsigned)nzc;
    env->cylinders = nullptr;
    env->num_cylinders = 0;
    env->cuboids = b;
    env->num_cuboids = (unsigned)ncb;
    env->z_aligned_cuboids = zb;
    env->num_z_aligned_cuboids = (unsigned)nzb;
}

