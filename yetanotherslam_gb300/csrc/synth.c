/*
 * synth.c — seeded synthetic RGB-D sequences for tests and benchmarks.
 *
 * Scene: an axis-aligned box room (camera inside) with spheres and
 * axis-aligned cuboids, each with its own Lambertian albedo; the albedo is
 * modulated by a smooth texture fixed in world coordinates, so brightness is
 * view-independent (photometric tracking has gradients to work with).
 * Light: one point light near the ceiling plus ambient.  Depth: camera-frame
 * z of the nearest hit, Gaussian noise sigma = 1.5 mm * z^2 (z in metres),
 * 1 % of pixels zeroed, stored as uint16 millimetres.  Colour: uint8 RGB.
 * Trajectory: smooth, at most 2 cm and 1 degree per frame.
 * Coordinates: camera x right, y down, z forward; world y points down.
 *
 * Randomness is counter based (SplitMix64 of seed/frame/pixel), so every
 * frame and pixel is reproducible independently of thread count.
 *
 * Multi-room variant (yas_synth_scene_init_rooms): a sx x sy x sz box split
 * into four rooms by two interior walls (planes x = 0 and z = 0, 0.1 m thick)
 * with a doorway wherever the loop path crosses a wall; objects avoid walls,
 * doorways and the path.  Its trajectory is a closed loop of radius
 * loop_radius around the vertical axis that returns to its start after
 * loop_frames frames, looking 0.9 rad outward from the direction of travel.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define SYN_MAX_OBJ 256

typedef struct {
    int kind; /* 0 sphere, 1 cuboid */
    double c[3], r;
    double lo[3], hi[3];
    double albedo[3];
} syn_obj;

typedef struct {
    int n_obj;
    syn_obj obj[SYN_MAX_OBJ];
    double room_lo[3], room_hi[3];
    double wall_albedo[6][3];
    double light[3];
    double tex_freq;
    double path_centre[3];
    double path_radius[3];
    int traj_kind; /* 0 figure-eight in the path box, 1 closed loop */
    int loop_frames;
    double loop_radius, loop_height;
    uint64_t seed;
} syn_scene;

static uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

static double u01(uint64_t *s) {
    *s = splitmix64(*s);
    return (double)(*s >> 11) * (1.0 / 9007199254740992.0);
}

static double urange(uint64_t *s, double a, double b) { return a + (b - a) * u01(s); }

int yas_synth_scene_size(void) { return (int)sizeof(syn_scene); }

/* Distance from point p to the camera path region (an axis-aligned box). */
static double dist_to_path(const syn_scene *sc, const double p[3]) {
    double d2 = 0.0;
    for (int i = 0; i < 3; ++i) {
        double lo = sc->path_centre[i] - sc->path_radius[i], hi = sc->path_centre[i] + sc->path_radius[i];
        double d = p[i] < lo ? lo - p[i] : (p[i] > hi ? p[i] - hi : 0.0);
        d2 += d * d;
    }
    return sqrt(d2);
}

/* Room of size (sx, sy, sz) metres centred at the origin; n_spheres spheres of
 * radius U[0.1, 0.5] m and n_boxes cuboids of side U[0.1, 0.6] m. */
int yas_synth_scene_init(syn_scene *sc, uint64_t seed, int n_spheres, int n_boxes, double sx, double sy,
                         double sz) {
    if (n_spheres + n_boxes > SYN_MAX_OBJ) return 1;
    memset(sc, 0, sizeof(*sc));
    sc->seed = seed;
    uint64_t s = splitmix64(seed ^ 0x5CE4E5B9ULL);
    sc->room_lo[0] = -sx / 2;
    sc->room_hi[0] = sx / 2;
    sc->room_lo[1] = -sy / 2;
    sc->room_hi[1] = sy / 2;
    sc->room_lo[2] = -sz / 2;
    sc->room_hi[2] = sz / 2;
    for (int f = 0; f < 6; ++f)
        for (int c = 0; c < 3; ++c) sc->wall_albedo[f][c] = urange(&s, 0.35, 0.9);
    sc->light[0] = 0.3;
    sc->light[1] = sc->room_lo[1] + 0.1;
    sc->light[2] = 0.2;
    sc->tex_freq = 2.0 * 3.14159265358979323846 / 0.25;
    sc->path_centre[0] = 0.0;
    sc->path_centre[1] = 0.0;
    sc->path_centre[2] = -0.35 * sz / 2;
    sc->path_radius[0] = 0.45;
    sc->path_radius[1] = 0.15;
    sc->path_radius[2] = 0.35;
    int placed = 0, tries = 0;
    while (placed < n_spheres + n_boxes && tries < 100000) {
        ++tries;
        syn_obj o;
        memset(&o, 0, sizeof(o));
        o.kind = placed < n_spheres ? 0 : 1;
        for (int c = 0; c < 3; ++c) o.albedo[c] = urange(&s, 0.2, 1.0);
        if (o.kind == 0) {
            o.r = urange(&s, 0.1, 0.5);
            for (int i = 0; i < 3; ++i) o.c[i] = urange(&s, sc->room_lo[i] + o.r, sc->room_hi[i] - o.r);
            if (dist_to_path(sc, o.c) < o.r + 0.45) continue;
        } else {
            double half[3], cen[3];
            for (int i = 0; i < 3; ++i) half[i] = 0.5 * urange(&s, 0.1, 0.6);
            for (int i = 0; i < 3; ++i) cen[i] = urange(&s, sc->room_lo[i] + half[i], sc->room_hi[i] - half[i]);
            /* about half the cuboids rest on the floor (world +y is down) */
            if (u01(&s) < 0.5) cen[1] = sc->room_hi[1] - half[1];
            double rad = sqrt(half[0] * half[0] + half[1] * half[1] + half[2] * half[2]);
            if (dist_to_path(sc, cen) < rad + 0.45) continue;
            for (int i = 0; i < 3; ++i) {
                o.lo[i] = cen[i] - half[i];
                o.hi[i] = cen[i] + half[i];
            }
        }
        sc->obj[placed++] = o;
    }
    sc->n_obj = placed;
    return placed == n_spheres + n_boxes ? 0 : 2;
}

/* Distance from p to the loop path (a horizontal circle) in the x-z plane and
 * in height. */
static double dist_to_loop(const syn_scene *sc, const double p[3]) {
    const double rr = sqrt(p[0] * p[0] + p[2] * p[2]);
    const double dr = rr - sc->loop_radius, dy = p[1] - sc->loop_height;
    return sqrt(dr * dr + dy * dy);
}

static void add_box(syn_scene *sc, const double lo[3], const double hi[3], const double alb[3]) {
    syn_obj o;
    memset(&o, 0, sizeof(o));
    o.kind = 1;
    for (int i = 0; i < 3; ++i) {
        o.lo[i] = lo[i];
        o.hi[i] = hi[i];
        o.albedo[i] = alb[i];
    }
    sc->obj[sc->n_obj++] = o;
}

/* Four rooms in an sx x sy x sz box (y is height, +y down); n_objects
 * spheres and cuboids (half each) with the radii / sides of the single-room
 * scene; a closed loop of radius `radius` metres, `frames` frames long. */
int yas_synth_scene_init_rooms(syn_scene *sc, uint64_t seed, int n_objects, double sx, double sy, double sz,
                               double radius, int frames) {
    if (n_objects + 8 > SYN_MAX_OBJ || frames < 8 || radius <= 0.5 || radius >= 0.5 * sx || radius >= 0.5 * sz)
        return 1;
    memset(sc, 0, sizeof(*sc));
    sc->seed = seed;
    uint64_t s = splitmix64(seed ^ 0x9E0D2C1BULL);
    sc->room_lo[0] = -sx / 2;
    sc->room_hi[0] = sx / 2;
    sc->room_lo[1] = -sy / 2;
    sc->room_hi[1] = sy / 2;
    sc->room_lo[2] = -sz / 2;
    sc->room_hi[2] = sz / 2;
    for (int f = 0; f < 6; ++f)
        for (int c = 0; c < 3; ++c) sc->wall_albedo[f][c] = urange(&s, 0.35, 0.9);
    sc->light[0] = 0.3;
    sc->light[1] = sc->room_lo[1] + 0.1;
    sc->light[2] = 0.2;
    sc->tex_freq = 2.0 * 3.14159265358979323846 / 0.25;
    sc->traj_kind = 1;
    sc->loop_frames = frames;
    sc->loop_radius = radius;
    sc->loop_height = 0.1 * sy / 2;
    /* interior walls: x = 0 (along z) and z = 0 (along x), each cut by two
     * doorways centred where the loop crosses it: 1.4 m wide, up to 2.6 m */
    const double th = 0.05, door = 0.7, floor_y = sc->room_hi[1], top_y = sc->room_lo[1];
    const double door_top = floor_y - 2.6;
    for (int w = 0; w < 2; ++w) {
        const int along = w == 0 ? 2 : 0, across = w == 0 ? 0 : 2;
        double alb[3];
        for (int c = 0; c < 3; ++c) alb[c] = urange(&s, 0.35, 0.9);
        /* segments along the wall: [lo, -r-door], [-r+door, r-door], [r+door, hi] */
        const double seg[3][2] = {{sc->room_lo[along], -radius - door},
                                  {-radius + door, radius - door},
                                  {radius + door, sc->room_hi[along]}};
        for (int k = 0; k < 3; ++k) {
            double lo[3], hi[3];
            lo[across] = -th;
            hi[across] = th;
            lo[1] = top_y;
            hi[1] = floor_y;
            lo[along] = seg[k][0];
            hi[along] = seg[k][1];
            add_box(sc, lo, hi, alb);
        }
        for (int k = 0; k < 2; ++k) { /* lintels over the doorways */
            double lo[3], hi[3];
            lo[across] = -th;
            hi[across] = th;
            lo[1] = top_y;
            hi[1] = door_top;
            const double c = k == 0 ? -radius : radius;
            lo[along] = c - door;
            hi[along] = c + door;
            add_box(sc, lo, hi, alb);
        }
    }
    const int n_walls = sc->n_obj;
    int placed = 0, tries = 0;
    while (placed < n_objects && tries < 200000) {
        ++tries;
        syn_obj o;
        memset(&o, 0, sizeof(o));
        o.kind = placed < n_objects / 2 ? 0 : 1;
        for (int c = 0; c < 3; ++c) o.albedo[c] = urange(&s, 0.2, 1.0);
        double cen[3], rad;
        if (o.kind == 0) {
            o.r = urange(&s, 0.1, 0.5);
            for (int i = 0; i < 3; ++i) cen[i] = urange(&s, sc->room_lo[i] + o.r, sc->room_hi[i] - o.r);
            rad = o.r;
            for (int i = 0; i < 3; ++i) o.c[i] = cen[i];
        } else {
            double half[3];
            for (int i = 0; i < 3; ++i) half[i] = 0.5 * urange(&s, 0.1, 0.6);
            for (int i = 0; i < 3; ++i) cen[i] = urange(&s, sc->room_lo[i] + half[i], sc->room_hi[i] - half[i]);
            if (u01(&s) < 0.5) cen[1] = sc->room_hi[1] - half[1];
            rad = sqrt(half[0] * half[0] + half[1] * half[1] + half[2] * half[2]);
            for (int i = 0; i < 3; ++i) {
                o.lo[i] = cen[i] - half[i];
                o.hi[i] = cen[i] + half[i];
            }
        }
        /* clear of the interior walls and of the path */
        if (fabs(cen[0]) < rad + th + 0.05 || fabs(cen[2]) < rad + th + 0.05) continue;
        if (dist_to_loop(sc, cen) < rad + 0.6) continue;
        sc->obj[sc->n_obj++] = o;
        ++placed;
    }
    return placed == n_objects && sc->n_obj == n_walls + n_objects ? 0 : 2;
}

/* Camera-to-world pose (row-major 3x4) of frame `i`: a smooth figure-eight
 * inside the path box with slowly varying yaw and pitch.  Per-frame motion is
 * below 2 cm and 1 degree. */
static void loop_pose(const syn_scene *sc, int i, double out[12]) {
    const double two_pi = 2.0 * 3.14159265358979323846;
    const double th = two_pi * (double)i / (double)sc->loop_frames;
    const double R = sc->loop_radius;
    const double px = R * cos(th), pz = R * sin(th);
    const double py = sc->loop_height + 0.05 * sin(3.0 * th);
    /* the camera's z axis 0.9 rad outward from the path's tangent
     * (-sin th, 0, cos th), towards the outer walls, with a gentle sway; yaw
     * about world y, then pitch, then roll */
    const double yaw = -th + 0.9 + 0.15 * sin(5.0 * th);
    const double pitch = 0.08 * sin(4.0 * th);
    const double roll = 0.03 * sin(7.0 * th);
    const double cy = cos(yaw), sy = sin(yaw), cp = cos(pitch), sp = sin(pitch), cr = cos(roll), sr = sin(roll);
    const double Ry[9] = {cy, 0, sy, 0, 1, 0, -sy, 0, cy};
    const double Rx[9] = {1, 0, 0, 0, cp, -sp, 0, sp, cp};
    const double Rz[9] = {cr, -sr, 0, sr, cr, 0, 0, 0, 1};
    double A[9], Rm[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            A[r * 3 + c] = Ry[r * 3 + 0] * Rx[0 * 3 + c] + Ry[r * 3 + 1] * Rx[1 * 3 + c] + Ry[r * 3 + 2] * Rx[2 * 3 + c];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            Rm[r * 3 + c] = A[r * 3 + 0] * Rz[0 * 3 + c] + A[r * 3 + 1] * Rz[1 * 3 + c] + A[r * 3 + 2] * Rz[2 * 3 + c];
    for (int r = 0; r < 3; ++r) {
        out[r * 4 + 0] = Rm[r * 3 + 0];
        out[r * 4 + 1] = Rm[r * 3 + 1];
        out[r * 4 + 2] = Rm[r * 3 + 2];
    }
    out[3] = px;
    out[7] = py;
    out[11] = pz;
}

void yas_synth_pose(const syn_scene *sc, int i, double out[12]) {
    if (sc->traj_kind == 1) {
        loop_pose(sc, i, out);
        return;
    }
    const double w = 0.021;
    const double t = (double)i;
    const double px = sc->path_centre[0] + sc->path_radius[0] * sin(w * t);
    const double py = sc->path_centre[1] + sc->path_radius[1] * sin(1.7 * w * t);
    const double pz = sc->path_centre[2] + sc->path_radius[2] * sin(2.0 * w * t);
    const double yaw = 0.45 * sin(0.6 * w * t + 0.3);
    const double pitch = 0.12 * sin(1.3 * w * t);
    const double roll = 0.05 * sin(0.9 * w * t);
    const double cy = cos(yaw), sy = sin(yaw), cp = cos(pitch), sp = sin(pitch), cr = cos(roll), sr = sin(roll);
    /* R = Ry(yaw) * Rx(pitch) * Rz(roll) */
    const double Ry[9] = {cy, 0, sy, 0, 1, 0, -sy, 0, cy};
    const double Rx[9] = {1, 0, 0, 0, cp, -sp, 0, sp, cp};
    const double Rz[9] = {cr, -sr, 0, sr, cr, 0, 0, 0, 1};
    double A[9], R[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            A[r * 3 + c] = Ry[r * 3 + 0] * Rx[0 * 3 + c] + Ry[r * 3 + 1] * Rx[1 * 3 + c] + Ry[r * 3 + 2] * Rx[2 * 3 + c];
        }
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            R[r * 3 + c] = A[r * 3 + 0] * Rz[0 * 3 + c] + A[r * 3 + 1] * Rz[1 * 3 + c] + A[r * 3 + 2] * Rz[2 * 3 + c];
        }
    for (int r = 0; r < 3; ++r) {
        out[r * 4 + 0] = R[r * 3 + 0];
        out[r * 4 + 1] = R[r * 3 + 1];
        out[r * 4 + 2] = R[r * 3 + 2];
    }
    out[3] = px;
    out[7] = py;
    out[11] = pz;
}

/* Nearest hit along o + t d (t > 1e-6): returns t, fills normal and albedo.
 * Only the objects whose bit is set in `cand` (NULL: all) are tested, in
 * index order, so a conservative candidate set gives the brute-force hit. */
static double trace(const syn_scene *sc, const double o[3], const double d[3], double n[3], double alb[3],
                    const uint64_t *cand) {
    double best = 1e30;
    /* room: exit distance from inside */
    for (int a = 0; a < 3; ++a) {
        if (d[a] == 0.0) continue;
        double bound = d[a] > 0 ? sc->room_hi[a] : sc->room_lo[a];
        double t = (bound - o[a]) / d[a];
        if (t > 1e-6 && t < best) {
            best = t;
            n[0] = n[1] = n[2] = 0.0;
            n[a] = d[a] > 0 ? -1.0 : 1.0;
            int face = 2 * a + (d[a] > 0 ? 1 : 0);
            for (int c = 0; c < 3; ++c) alb[c] = sc->wall_albedo[face][c];
        }
    }
    for (int k = 0; k < sc->n_obj; ++k) {
        if (cand && !((cand[k >> 6] >> (k & 63)) & 1u)) continue;
        const syn_obj *ob = &sc->obj[k];
        if (ob->kind == 0) {
            double oc[3] = {o[0] - ob->c[0], o[1] - ob->c[1], o[2] - ob->c[2]};
            double a = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            double b = 2.0 * (oc[0] * d[0] + oc[1] * d[1] + oc[2] * d[2]);
            double c = oc[0] * oc[0] + oc[1] * oc[1] + oc[2] * oc[2] - ob->r * ob->r;
            double disc = b * b - 4 * a * c;
            if (disc < 0) continue;
            double sq = sqrt(disc);
            double t = (-b - sq) / (2 * a);
            if (t <= 1e-6) t = (-b + sq) / (2 * a);
            if (t > 1e-6 && t < best) {
                best = t;
                for (int i = 0; i < 3; ++i) n[i] = (o[i] + t * d[i] - ob->c[i]) / ob->r;
                for (int i = 0; i < 3; ++i) alb[i] = ob->albedo[i];
            }
        } else {
            double tmin = -1e30, tmax = 1e30;
            int amin = 0;
            int ok = 1;
            for (int a = 0; a < 3 && ok; ++a) {
                if (d[a] == 0.0) {
                    if (o[a] < ob->lo[a] || o[a] > ob->hi[a]) ok = 0;
                    continue;
                }
                double t1 = (ob->lo[a] - o[a]) / d[a], t2 = (ob->hi[a] - o[a]) / d[a];
                if (t1 > t2) {
                    double tt = t1;
                    t1 = t2;
                    t2 = tt;
                }
                if (t1 > tmin) {
                    tmin = t1;
                    amin = a;
                }
                if (t2 < tmax) tmax = t2;
            }
            if (!ok || tmin > tmax || tmin <= 1e-6) continue;
            if (tmin < best) {
                best = tmin;
                n[0] = n[1] = n[2] = 0.0;
                n[amin] = d[amin] > 0 ? -1.0 : 1.0;
                for (int i = 0; i < 3; ++i) alb[i] = ob->albedo[i];
            }
        }
    }
    return best;
}

static double gauss(uint64_t key) {
    uint64_t s = key;
    double u1 = u01(&s), u2 = u01(&s);
    if (u1 < 1e-300) u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * 3.14159265358979323846 * u2);
}

#define SYN_TILE 16
#define SYN_WORDS (SYN_MAX_OBJ / 64)

/* Screen rectangle (pixels, inclusive, clamped) that contains every pixel
 * whose ray can hit object `ob`: the bounds of its world AABB's projected
 * corners, widened by two pixels; the whole screen when a corner is not in
 * front of the camera.  Returns 0 when the object is entirely behind it. */
static int object_rect(const syn_obj *ob, const double Twc[12], int w, int h, double fx, double fy, double cx,
                       double cy, int rect[4]) {
    double lo[3], hi[3];
    for (int i = 0; i < 3; ++i) {
        lo[i] = ob->kind == 0 ? ob->c[i] - ob->r : ob->lo[i];
        hi[i] = ob->kind == 0 ? ob->c[i] + ob->r : ob->hi[i];
    }
    double umin = 1e30, umax = -1e30, vmin = 1e30, vmax = -1e30;
    int behind = 0, front = 0;
    for (int c = 0; c < 8; ++c) {
        const double p[3] = {(c & 1) ? hi[0] : lo[0], (c & 2) ? hi[1] : lo[1], (c & 4) ? hi[2] : lo[2]};
        const double q[3] = {p[0] - Twc[3], p[1] - Twc[7], p[2] - Twc[11]};
        /* camera frame: R^T (p - t) */
        const double x = Twc[0] * q[0] + Twc[4] * q[1] + Twc[8] * q[2];
        const double y = Twc[1] * q[0] + Twc[5] * q[1] + Twc[9] * q[2];
        const double z = Twc[2] * q[0] + Twc[6] * q[1] + Twc[10] * q[2];
        if (z <= 1e-3) {
            ++behind;
            continue;
        }
        ++front;
        const double u = fx * x / z + cx, v = fy * y / z + cy;
        umin = u < umin ? u : umin;
        umax = u > umax ? u : umax;
        vmin = v < vmin ? v : vmin;
        vmax = v > vmax ? v : vmax;
    }
    if (!front) return 0;
    if (behind) {
        rect[0] = 0, rect[1] = 0, rect[2] = w - 1, rect[3] = h - 1;
        return 1;
    }
    const double u0 = floor(umin) - 2, u1 = ceil(umax) + 2, v0 = floor(vmin) - 2, v1 = ceil(vmax) + 2;
    if (u1 < 0 || v1 < 0 || u0 > w - 1 || v0 > h - 1) return 0;
    rect[0] = u0 < 0 ? 0 : (int)u0;
    rect[1] = v0 < 0 ? 0 : (int)v0;
    rect[2] = u1 > w - 1 ? w - 1 : (int)u1;
    rect[3] = v1 > h - 1 ? h - 1 : (int)v1;
    return 1;
}

static void render_impl(const syn_scene *sc, const double Twc[12], int w, int h, double fx, double fy, double cx,
                        double cy, int frame, uint8_t *rgb, uint16_t *depth, float *clean, int cull) {
    const double o[3] = {Twc[3], Twc[7], Twc[11]};
    /* per 16x16 tile, the objects that can appear in it */
    const int tw = (w + SYN_TILE - 1) / SYN_TILE, tht = (h + SYN_TILE - 1) / SYN_TILE;
    uint64_t *tiles = NULL;
    if (cull) {
        tiles = (uint64_t *)calloc((size_t)tw * tht * SYN_WORDS, sizeof(uint64_t));
        if (!tiles) cull = 0;
    }
    if (cull) {
        for (int k = 0; k < sc->n_obj; ++k) {
            int r[4];
            if (!object_rect(&sc->obj[k], Twc, w, h, fx, fy, cx, cy, r)) continue;
            for (int ty = r[1] / SYN_TILE; ty <= r[3] / SYN_TILE; ++ty)
                for (int tx = r[0] / SYN_TILE; tx <= r[2] / SYN_TILE; ++tx)
                    tiles[((size_t)ty * tw + tx) * SYN_WORDS + (k >> 6)] |= 1ull << (k & 63);
        }
    }
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            const double dc[3] = {(x - cx) / fx, (y - cy) / fy, 1.0};
            double d[3];
            for (int r = 0; r < 3; ++r) d[r] = Twc[r * 4 + 0] * dc[0] + Twc[r * 4 + 1] * dc[1] + Twc[r * 4 + 2] * dc[2];
            double n[3] = {0, 0, 0}, alb[3] = {0, 0, 0};
            const uint64_t *cand =
                cull ? tiles + ((size_t)(y / SYN_TILE) * tw + (size_t)(x / SYN_TILE)) * SYN_WORDS : NULL;
            const double t = trace(sc, o, d, n, alb, cand);
            const size_t k = (size_t)y * w + x;
            const int hit = t < 1e29;
            if (clean) clean[k] = hit ? (float)t : 0.0f;
            if (depth) {
                uint16_t v = 0;
                if (hit) {
                    const uint64_t key = splitmix64(sc->seed ^ splitmix64(((uint64_t)frame << 32) ^ (uint64_t)k));
                    uint64_t s2 = key ^ 0xD1B54A32D192ED03ULL;
                    const double drop = u01(&s2);
                    const double z = t + 0.0015 * t * t * gauss(key);
                    const double mm = floor(z * 1000.0 + 0.5);
                    if (drop >= 0.01 && mm > 0.0 && mm < 65535.0) v = (uint16_t)mm;
                }
                depth[k] = v;
            }
            if (rgb) {
                double shade = 0.0;
                if (hit) {
                    const double p[3] = {o[0] + t * d[0], o[1] + t * d[1], o[2] + t * d[2]};
                    double l[3] = {sc->light[0] - p[0], sc->light[1] - p[1], sc->light[2] - p[2]};
                    const double ln = sqrt(l[0] * l[0] + l[1] * l[1] + l[2] * l[2]);
                    const double ndl = (n[0] * l[0] + n[1] * l[1] + n[2] * l[2]) / (ln > 0 ? ln : 1.0);
                    const double f = sc->tex_freq;
                    const double tex = 0.7 + 0.15 * sin(f * p[0]) * cos(0.8 * f * p[1]) + 0.15 * sin(0.9 * f * p[2] + 1.3 * f * p[0]);
                    shade = (0.3 + 0.7 * (ndl > 0 ? ndl : 0.0)) * tex;
                }
                for (int c = 0; c < 3; ++c) {
                    double v = alb[c] * shade * 255.0;
                    v = v < 0 ? 0 : (v > 255 ? 255 : v);
                    rgb[k * 3 + c] = (uint8_t)floor(v + 0.5);
                }
            }
        }
    }
    free(tiles);
}

/* Renders one frame at camera-to-world pose Twc.  rgb: w*h*3 (may be NULL),
 * depth: w*h uint16 mm (may be NULL), clean: w*h float metres without noise
 * or dropout (may be NULL). */
void yas_synth_render(const syn_scene *sc, const double Twc[12], int w, int h, double fx, double fy, double cx,
                      double cy, int frame, uint8_t *rgb, uint16_t *depth, float *clean) {
    render_impl(sc, Twc, w, h, fx, fy, cx, cy, frame, rgb, depth, clean, 1);
}

/* The same without the per-tile object lists (every object tested for every
 * pixel): the reference the culled renderer must match bit for bit. */
void yas_synth_render_brute(const syn_scene *sc, const double Twc[12], int w, int h, double fx, double fy,
                            double cx, double cy, int frame, uint8_t *rgb, uint16_t *depth, float *clean) {
    render_impl(sc, Twc, w, h, fx, fy, cx, cy, frame, rgb, depth, clean, 0);
}
