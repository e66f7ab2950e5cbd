/*
 * rt_types.h: base scalar/vector typedefs of the QuadRay scene API.
 *
 * The scene-description structs (format.h) and the engine API (engine.h)
 * are written against these names so that scene data authored for the
 * reference engine (VectorChief/QuadRay-engine, core/config/rtbase.h:574-736)
 * compiles unchanged.  Only the fp32 build is provided: the render path
 * computes in single precision like the reference's RT_ELEMENT=32 build.
 */
#ifndef QR_RT_TYPES_H
#define QR_RT_TYPES_H

#include <stdint.h>
#include <stddef.h>
#include <float.h>

typedef void                rt_void;
typedef void               *rt_pntr;
typedef char               *rt_pstr;
typedef int8_t              rt_si08;
typedef uint8_t             rt_ui08;
typedef int16_t             rt_si16;
typedef uint16_t            rt_ui16;
typedef int32_t             rt_si32;
typedef uint32_t            rt_ui32;
typedef int64_t             rt_si64;
typedef uint64_t            rt_ui64;
typedef rt_si08             rt_bool;
typedef rt_si64             rt_time;
typedef rt_si64             rt_cell;
typedef rt_si64             rt_size;
typedef rt_ui64             rt_word;
typedef rt_si32             rt_elem;
typedef rt_ui32             rt_uelm;

typedef float               rt_fp32;
typedef double              rt_fp64;
typedef rt_fp32             rt_real;
typedef rt_fp32             rt_vec2[2];
typedef rt_fp32             rt_vec3[3];
typedef rt_fp32             rt_vec4[4];
typedef rt_fp32             rt_mat4[4][4];

#define RT_NULL             0
#define RT_TRUE             1
#define RT_FALSE            0

#define RT_ARR_SIZE(a)      (sizeof(a) / sizeof((a)[0]))

/* largest finite fp32, used by the reference as "infinity" for clip boxes
 * and depth limits (core/config/rtbase.h:823, 932) */
#define RT_INF              (FLT_MAX)
#define RT_PI               (3.14159265358979323846)

/* axis indices (core/config/rtbase.h:793-801) */
#define RT_X                0
#define RT_Y                1
#define RT_Z                2
#define RT_W                3
#define RT_I                0
#define RT_J                1
#define RT_K                2
#define RT_L                3
#define RT_U                0
#define RT_V                1
#define RT_R                0
#define RT_G                1
#define RT_B                2
#define RT_A                3

#define RT_MIN(a, b)        ((a) < (b) ? (a) : (b))
#define RT_MAX(a, b)        ((a) > (b) ? (a) : (b))

#endif /* QR_RT_TYPES_H */
