"""Independent pure-Python restatement of simuverse's reference-mode D2Q9 step (test code).

Written separately from oracle/lbm_oracle.c and used only to generate the small golden
fixtures in this folder, which pin the C oracle and the CUDA kernels to the same
numbers.  Every float operation is done on numpy float32 scalars, so it rounds exactly
like the WGSL expression it restates (no multiply-add contraction).  Sources:
  init.wgsl:19-63, collide_stream.wgsl:25-88, boundary.wgsl:3-35,
  layout_and_fn.wgsl:38-51, d2q9_fn.wgsl:1-26, simuverse/src/fluid/mod.rs:39-52,
  simuverse/src/fluid/lattice.rs:26-98, simuverse/src/fluid/d2q9_node.rs:215-245.
Slow by design: lattices of a few hundred cells only.
"""
import numpy as np

f32 = np.float32
E = [(0, 0), (1, 0), (0, -1), (-1, 0), (0, 1), (1, -1), (-1, -1), (-1, 1), (1, 1)]
INV = [0, 3, 4, 1, 2, 7, 8, 5, 6]
W = [f32(0.444444)] + [f32(0.111111)] * 4 + [f32(0.0277777)] * 4
MAXV = [f32(0.6)] + [f32(0.2222)] * 4 + [f32(0.1111)] * 4
R_OBS = f32(28.0)


def mask(nx, ny, scene, lid=0.13, inlet=0.12):
    """lattice.rs:26-98 -> (material, block_iter, vx, vy) lists indexed [y][x]."""
    mat = [[1] * nx for _ in range(ny)]
    vx = [[f32(0.0)] * nx for _ in range(ny)]
    s = [(f32(nx) / f32(7.0) - R_OBS, f32(ny) / f32(2.0)), (f32(nx) / f32(5.0), f32(ny) / f32(4.0)),
         (f32(nx) / f32(5.0), f32(ny) * f32(0.75))]
    for y in range(ny):
        for x in range(nx):
            if scene == "custom":
                if x == 0 or x == nx - 1 or y == 0 or y == ny - 1:
                    mat[y][x] = 2
            elif scene == "cavity":
                if x == 0 or x == nx - 1 or y == ny - 1:
                    mat[y][x] = 2
                elif y == 0:
                    mat[y][x] = 7
                elif y == 1:
                    mat[y][x] = 6
                    vx[y][x] = f32(lid)
            else:
                if y == 0 or y == ny - 1:
                    mat[y][x] = 2
                elif x == 0 or x == nx - 1:
                    mat[y][x] = 7
                elif x == 1:
                    mat[y][x] = 3
                    vx[y][x] = f32(inlet)
                elif x == nx - 2:
                    mat[y][x] = 5
                else:
                    for sx, sy in s:
                        dx, dy = f32(x) - sx, f32(y) - sy
                        if np.sqrt(dx * dx + dy * dy, dtype=np.float32) <= R_OBS:
                            mat[y][x] = 4
    info = np.zeros((ny, nx), dtype=[("material", "<i4"), ("block_iter", "<i4"), ("vx", "<f4"), ("vy", "<f4")])
    for y in range(ny):
        for x in range(nx):
            info[y, x] = (mat[y][x], -1, vx[y][x], 0.0)
    return info


def solid(m):
    return m == 2 or m == 4


class PyRef:
    def __init__(self, info, tau, fluid_ty):
        self.info = info.copy()
        self.ny, self.nx = info.shape
        self.omega = f32(1.0) / f32(tau)
        ny, nx = self.ny, self.nx
        self.A = np.zeros((9, ny, nx), np.float32)
        self.B = np.zeros((9, ny, nx), np.float32)
        for y in range(ny):
            for x in range(nx):
                m = int(self.info[y, x]["material"])
                if solid(m):
                    continue
                for i in range(9):
                    self.A[i, y, x] = W[i]
                if fluid_ty == 0:
                    t = W[3] * f32(0.5)
                    self.A[1, y, x] = W[1] + t
                    self.A[3, y, x] = t
                    self.B[1, y, x] = W[1] + t
                    self.B[3, y, x] = t
                if m in (3, 6) and int(self.info[y, x]["block_iter"]) > 0:
                    self.info[y, x] = (1, 0, 0.0, 0.0)
        self.macro = np.zeros((ny, nx, 4), np.float32)
        self.macro[..., 3] = 1.0

    def step(self):
        nx, ny = self.nx, self.ny
        A, B = self.A, self.B
        for y in range(ny):
            for x in range(nx):
                rec = self.info[y, x]
                m = int(rec["material"])
                if solid(m):
                    self.macro[y, x] = 0.0
                    continue
                f = []
                rho, vx, vy = f32(0), f32(0), f32(0)
                for i in range(9):
                    ex, ey = E[INV[i]]
                    sx, sy = x + ex, y + ey
                    sx = nx - 1 if sx < 0 else (0 if sx >= nx else sx)
                    sy = ny - 1 if sy < 0 else (0 if sy >= ny else sy)
                    v = A[i, sy, sx]
                    f.append(v)
                    rho = rho + v
                    vx = vx + f32(E[i][0]) * v
                    vy = vy + f32(E[i][1]) * v
                rho = min(max(rho, f32(0.8)), f32(1.2))
                vx = vx / rho
                vy = vy / rho
                F = [f32(0)] * 9
                if m in (3, 6):
                    bi = int(rec["block_iter"])
                    if bi > 0:
                        bi -= 1
                        if bi == 0:
                            m = 1
                    self.info[y, x] = (m, bi, rec["vx"], rec["vy"])
                    fx, fy = f32(rec["vx"]), f32(rec["vy"])
                    vx = fx * f32(0.5) / rho
                    vy = fy * f32(0.5) / rho
                    F = [W[i] * f32(3.0) * (f32(E[i][0]) * fx + f32(E[i][1]) * fy) for i in range(9)]
                self.macro[y, x] = (vx, vy, rho, 1.0)
                usqr = f32(1.5) * (vx * vx + vy * vy)
                for i in range(9):
                    eu = f32(E[i][0]) * vx + f32(E[i][1]) * vy
                    feq = rho * W[i] * (f32(1.0) + f32(3.0) * eu + f32(4.5) * (eu * eu) - usqr)
                    t = f[i] - self.omega * (f[i] - feq) + F[i]
                    if t > MAXV[i]:
                        t = MAXV[i]
                    elif t < 0:
                        t = f32(0)
                    B[i, y, x] = t
        # boundary pass: read all moved values, write them, then write the zeros
        moves, zeros = [], []
        for y in range(ny):
            for x in range(nx):
                if not solid(int(self.info[y, x]["material"])):
                    continue
                for i in range(9):
                    nxp, nyp = x - E[i][0], y - E[i][1]
                    if nxp <= 0 or nyp <= 0 or nxp >= nx - 1 or nyp >= ny - 1:
                        continue
                    moves.append((INV[i], y, x, B[i, nyp, nxp]))
                    zeros.append((i, nyp, nxp))
        for i, y, x, v in moves:
            B[i, y, x] = v
        for i, y, x in zeros:
            B[i, y, x] = 0.0
        self.A, self.B = B, A

    def add_obstacle(self, host_info, x, y):
        """d2q9_node.rs:215-245 with the host copy host_info."""
        cx, cy = f32(x) + f32(0.5), f32(y) + f32(0.5)
        for yy in range(y - 28, y + 28):
            for xx in range(self.nx):
                dx, dy = f32(xx) + f32(0.5) - cx, f32(yy) + f32(0.5) - cy
                if np.sqrt(dx * dx + dy * dy, dtype=np.float32) <= R_OBS:
                    host_info[yy, xx] = (4, -1, 0.0, 0.0)
                self.info[yy, xx] = host_info[yy, xx]
