"""Writes up_sinnet_data.h: the weight tables of the two sine-network shapes
(bunny, monkey head) of the reference's sources/sdf.cpp:252-290, read from
the reference project's source tree, whose root is the one required argument.
The tables define the shapes, so they are kept alike; the header is committed
and this recipe only regenerates it.

  python gen_sinnet_data.py <reference_root>
"""
import re
import sys
from pathlib import Path

if len(sys.argv) != 2:
    sys.exit("usage: python gen_sinnet_data.py <reference_root>  (the root of the unnatural-planets source tree)")
ROOT = Path(sys.argv[1])
src = (ROOT / 'sources' / 'sdf.cpp').read_text()
NUM = r'-?(?:\d+\.\d*|\.\d+|\d+)'
def vec4s(s): return [[float(x) for x in re.findall(NUM, m)] for m in re.findall(r'Vec4\(([^)]*)\)', s)]
def mat4s(s): return [[float(x) for x in re.findall(NUM, m)] for m in re.findall(r'Mat4\(([^)]*)\)', s)]
out = []
for name, key in [('bunny', 'sdfBunnyImpl'), ('monkey', 'sdfMonkeyHeadImpl')]:
    i = src.index('Real ' + key); j = src.index('return dot', i); k = src.index(';', j)
    body = src[i:k + 1]
    lines = [l.strip() for l in body.split('\n')]
    l0 = [l for l in lines if re.match(r'Vec4 f0?0?_?\d?\w* = sin\(p\[1\]', l)]
    assert len(l0) == 4, (name, len(l0))
    xsign = -1.0 if '- p[0]' in l0[0] else 1.0
    in_y, in_z, in_x, in_b = [], [], [], []
    for l in l0:
        v = vec4s(l); assert len(v) == 4
        in_y.append(v[0]); in_z.append(v[1]); in_x.append(v[2]); in_b.append(v[3])
    hid = [l for l in lines if 'Mat4(' in l]
    assert len(hid) == 8
    L = []
    for l in hid:
        m = mat4s(l); v = vec4s(l); assert len(m) == 4 and len(v) == 1
        div = float(re.search(r'/\s*(' + NUM + r')\s*\+', l).group(1))
        L.append((m, v[0], div))
    ret = [l for l in lines if l.startswith('return dot')][0]
    w = vec4s(ret); assert len(w) == 4
    mb = re.search(r'\)\)\s*([+-])\s*(' + NUM + r')\s*;', ret); bias = float(mb.group(2)) * (1 if mb.group(1) == '+' else -1)
    def arr(a): return '{' + ', '.join(repr(float(x)) + 'f' for x in a) + '}'
    out.append(f'// {name}: sources/sdf.cpp sine network (input {"minus" if xsign < 0 else "plus"} p.x term)')
    out.append(f'UP_SINNET_STORAGE SinNetWeights kSinNet_{name} = {{')
    out.append(f'\t{xsign}f,')
    out.append('\t{' + ', '.join(arr(r) for r in in_y) + '},')
    out.append('\t{' + ', '.join(arr(r) for r in in_z) + '},')
    out.append('\t{' + ', '.join(arr(r) for r in in_x) + '},')
    out.append('\t{' + ', '.join(arr(r) for r in in_b) + '},')
    out.append('\t{' + ', '.join('{' + ', '.join(arr(m) for m in L[q][0]) + '}' for q in range(8)) + '},')
    out.append('\t{' + ', '.join(arr(L[q][1]) for q in range(8)) + '},')
    out.append('\t{' + ', '.join(repr(L[q][2]) + 'f' for q in range(8)) + '},')
    out.append('\t{' + ', '.join(arr(r) for r in w) + '},')
    out.append(f'\t{bias}f,')
    out.append('};')
hdr = '''// Weights of the two sine-network shapes ("bunny" and "monkey head") of the
// reference's sources/sdf.cpp:252-290 (originally published on shadertoy,
// wtVyWK and wtdBzn). The shapes are defined by these numbers, so the table
// is kept alike; it is plain data shared by the CUDA path and the oracle.
//
// Network: f0[j] = sin(p.y*in_y[j] + p.z*in_z[j] + x_sign*p.x*in_x[j] + in_b[j])
//          f1[j] = sin(sum_m M[j][m] f0[m] + b[j]) / div[j] + f0[j]        (j = 0..3)
//          f2[j] = sin(sum_m M[4+j][m] f1[m] + b[4+j]) / div[4+j] + f1[j]
//          d     = sum_j dot(f2[j], out_w[j]) + out_b
// Each M is a 4x4 matrix stored column-major (16 floats): (M v)_r = sum_c M[4c+r] v_c.
#pragma once

// device code reads the tables from constant memory; host code (the oracle)
// from ordinary static data
#ifdef __CUDACC__
#define UP_SINNET_STORAGE static __constant__ const
#else
#define UP_SINNET_STORAGE static const
#endif

struct SinNetWeights {
	float x_sign;
	float in_y[4][4], in_z[4][4], in_x[4][4], in_b[4][4];
	float M[8][4][16];
	float b[8][4];
	float div[8];
	float out_w[4][4];
	float out_b;
};

'''
(Path(__file__).resolve().parent / 'up_sinnet_data.h').write_text(hdr + '\n'.join(out) + '\n')
print('ok')
