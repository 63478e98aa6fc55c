/* Body of the CPU restatement of the cuSten stencil kernels, instantiated for double and float by
 * stencil_oracle.c (REAL, FMA, SFX are defined there). Test infrastructure only.
 *
 * The restatement follows the reference kernels block by block and thread by thread:
 *   - a shared-memory tile of (BY+T+B) x (BX+L+R) per block, filled with the halo regions the
 *     reference loads for that block position (cuSten/src/kernels/2d_x_p_kernel.cu:100-150,
 *     2d_x_np_kernel.cu:97-176, 2d_y_p_kernel.cu:104-190, 2d_y_np_kernel.cu:104-250,
 *     2d_xy_p_kernel.cu:127-499, 2d_xy_np_kernel.cu:136-958 and the *_fun_kernel.cu twins);
 *     cells the reference never loads hold NaN;
 *   - per thread, the FMA chain in weight order from sum = 0 (2d_xy_p_kernel.cu:507-520), or the
 *     user function at the reference's index convention (X centre, Y centre + row stride, XY top-left
 *     + row stride + window size);
 *   - the reference's per-block write rules.
 * The Y non-periodic last block has no barrier between its loads and its reads in the reference
 * (2d_y_np_kernel.cu:227-249); the restatement computes what that block computes when the loads
 * complete first. */

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)

static REAL CAT(cube_minus_, SFX)(REAL c) { return FMA(c * c, c, -c); }

/* The six shipped device functions (custen_gb300/csrc/builtin_funs.cu), same operation order. */
static REAL CAT(fun_eval_, SFX)(int id, const REAL* d, const REAL* coe, int idx, int jump, int H, int V) {
    REAL s = (REAL)0;
    int k, j, i, count = 0;
    switch (id) {
    case 0: { REAL t = FMA((REAL)-2, d[idx], d[idx - 1]); t = t + d[idx + 1]; return t * coe[0]; }
    case 1: for (k = 0; k < 5; ++k) s = FMA(coe[k], CAT(cube_minus_, SFX)(d[idx - 2 + k]), s); return s;
    case 2: for (k = 0; k < 9; ++k) s = FMA(coe[k], d[(idx - 4 * jump) + k * jump], s); return s;
    case 3: for (k = 0; k < 5; ++k) s = FMA(coe[k], CAT(cube_minus_, SFX)(d[idx + (k - 2) * jump]), s); return s;
    case 4:
        for (j = 0; j < V; ++j)
            for (i = 0; i < H; ++i) s = FMA(coe[count++], d[idx + j * jump + i], s);
        return s;
    case 5:
        for (j = 0; j < V; ++j)
            for (i = 0; i < H; ++i) s = FMA(coe[count++], CAT(cube_minus_, SFX)(d[idx + j * jump + i]), s);
        return s;
    }
    return (REAL)NAN;
}

/* One Compute of `variant` over an nx x ny field split into numTiles tiles.
 * out:      updated in place; points the reference does not write keep their values.
 * in:       input field (tiles contiguous, tile t at in + t*nyTile*nx).
 * halo_src: base from which the per-tile halo pointers are derived with the periodic formulas of
 *           Create/Swap (custenCreateDestroy2DYp.cu:182-216); NULL means `in`.
 * coef:     weights (plain) or coefficients (Fun), ncoef of them.
 * fun_id:   shipped device function for the Fun variants (see above).
 * status:   per point 0 untouched, 1 written, 2 written from shared memory the reference never loaded
 *           (its value is undefined in the reference).
 * Returns 0, or -1 when the configuration is outside the reference's contract. */
int CAT(oracle_stencil_, SFX)(int variant, int nx, int ny, int numTiles, int BX, int BY, REAL* out, const REAL* in,
                              const REAL* halo_src, const REAL* coef, int ncoef, int H, int L, int R, int V, int T,
                              int B, int fun_id, unsigned char* status) {
    const int dir = variant < 4 ? 0 : (variant < 8 ? 1 : 2);
    const int fun = (variant == 2 || variant == 3 || variant == 6 || variant == 7 || variant == 10 || variant == 11);
    const int periodic = (variant == 0 || variant == 2 || variant == 4 || variant == 6 || variant == 8 || variant == 10);
    if (numTiles < 1 || ny % numTiles) return -1;
    const int nyTile = ny / numTiles;
    if (nx % BX || nyTile % BY) return -1;
    const int nbx = nx / BX, nby = nyTile / BY;
    if (dir != 1 && nbx < 2) return -1;                   /* both edge branches would run */
    if (dir != 0 && nby < 2) return -1;
    if (L > BX || R > BX || T > BY || B > BY) return -1;  /* halo loads cover at most one block */
    if (!halo_src) halo_src = in;
    const int nxL = BX + L + R, nyL = BY + T + B;
    REAL* sm = (REAL*)malloc(sizeof(REAL) * nxL * nyL);
    REAL coe_s[4096];
    if (!sm || ncoef > 4096) { free(sm); return -1; }
    for (int k = 0; k < ncoef; ++k) coe_s[k] = coef[k];

    for (int t = 0; t < numTiles; ++t) {
        const REAL* tile = in + (size_t)t * nyTile * nx;
        REAL* otile = out + (size_t)t * nyTile * nx;
        unsigned char* stile = status + (size_t)t * nyTile * nx;
        const int tileTop = (t == 0), tileBottom = (t == numTiles - 1);
        /* per-tile halo pointers (periodic formulas; only non-edge ones are read by np kernels) */
        const REAL* btop = halo_src + (size_t)((t == 0) ? (ny - T) : (t * nyTile - T)) * nx;
        const REAL* bbot = halo_src + (size_t)((t == numTiles - 1) ? 0 : (t + 1) * nyTile) * nx;
        for (int byi = 0; byi < nby; ++byi) {
            for (int bxi = 0; bxi < nbx; ++bxi) {
                const int bx0 = bxi * BX, by0 = byi * BY;
                const int left = (bxi == 0), right = (bxi == nbx - 1);
                const int topb = (byi == 0), botb = (byi == nby - 1);
                /* column sources: 0 none, 1 in-row, 2 wrap */
                int colL = left ? (periodic ? 2 : 0) : 1;
                int colR = right ? (periodic ? 2 : 0) : 1;
                /* row sources: 0 none, 1 tile rows, 2 halo pointer */
                int rowT = topb ? ((periodic || !tileTop) ? 2 : 0) : 1;
                int rowB = botb ? ((periodic || !tileBottom) ? 2 : 0) : 1;
                if (dir == 0) rowT = rowB = 0;
                if (dir == 1) colL = colR = 0;
                for (int k = 0; k < nxL * nyL; ++k) sm[k] = (REAL)NAN;
                for (int r = 0; r < nyL; ++r) {
                    int rsrc;
                    const REAL* rowp;
                    if (r < T) {
                        rsrc = rowT;
                        rowp = (rsrc == 1) ? tile + (size_t)(by0 - T + r) * nx : btop + (size_t)r * nx;
                    } else if (r < T + BY) {
                        rsrc = 1;
                        rowp = tile + (size_t)(by0 + r - T) * nx;
                    } else {
                        rsrc = rowB;
                        rowp = (rsrc == 1) ? tile + (size_t)(by0 + r - T) * nx : bbot + (size_t)(r - T - BY) * nx;
                    }
                    if (rsrc == 0) continue;
                    for (int c = 0; c < nxL; ++c) {
                        int x;
                        if (c < L) {
                            if (colL == 0) continue;
                            x = (colL == 1) ? bx0 - L + c : nx - L + c;
                        } else if (c < L + BX) {
                            x = bx0 + c - L;
                        } else {
                            if (colR == 0) continue;
                            x = (colR == 1) ? bx0 + c - L : c - L - BX;
                        }
                        sm[r * nxL + c] = rowp[x];
                    }
                }
                for (int ty = 0; ty < BY; ++ty) {
                    for (int tx = 0; tx < BX; ++tx) {
                        /* write rule of the reference block */
                        int act = 1; /* 0 skip, 1 write, 2 write zero */
                        if (variant == 1) {              /* Xnp */
                            if (left && tx < L) act = 0;
                            else if (right && tx >= BX - R) act = 2;
                        } else if (variant == 3) {       /* XnpFun */
                            if ((left && tx < L) || (right && tx >= BX - R)) act = 0;
                        } else if (variant == 5 || variant == 7) {   /* Ynp, YnpFun */
                            if ((topb && tileTop && ty < T) || (botb && tileBottom && ty >= BY - B)) act = 0;
                        } else if (variant == 9 || variant == 11) {  /* XYnp, XYnpFun */
                            int ok;
                            if (left && topb) ok = tileTop ? (tx >= L && ty >= T) : (tx >= L);
                            else if (right && topb) ok = tileTop ? (tx < BX - R && ty >= T) : (tx < BX - R);
                            else if (left && botb) ok = tileBottom ? (tx >= L && ty < BY - B) : (tx >= L);
                            else if (right && botb) ok = tileBottom ? (tx < BX - R && ty < BY - B) : (tx < BX - R);
                            else if (topb) ok = tileTop ? (ty >= T) : 1;
                            else if (botb) ok = tileBottom ? (ty < BY - B) : 1;
                            else if (left) ok = (tx >= L);
                            else if (right) ok = (tx < BX - L);   /* the reference guard (:862) */
                            else ok = 1;
                            act = ok ? 1 : 0;
                        }
                        if (act == 0) continue;
                        const size_t o = (size_t)(by0 + ty) * nx + (bx0 + tx);
                        if (act == 2) {
                            otile[o] = (REAL)0;
                            stile[o] = 1;
                            continue;
                        }
                        REAL v;
                        if (!fun) {
                            REAL sum = (REAL)0;
                            int w = 0;
                            for (int j = 0; j < V; ++j)
                                for (int i = 0; i < H; ++i) sum = FMA(coe_s[w++], sm[(ty + j) * nxL + tx + i], sum);
                            v = sum;
                        } else if (dir == 0) {
                            v = CAT(fun_eval_, SFX)(fun_id, sm, coe_s, ty * nxL + tx + L, 0, H, V);
                        } else if (dir == 1) {
                            v = CAT(fun_eval_, SFX)(fun_id, sm, coe_s, (ty + T) * nxL + tx + L, nxL, H, V);
                        } else {
                            v = CAT(fun_eval_, SFX)(fun_id, sm, coe_s, ty * nxL + tx, nxL, H, V);
                        }
                        otile[o] = v;
                        stile[o] = isnan(v) ? 2 : 1;
                    }
                }
            }
        }
    }
    free(sm);
    return 0;
}

#undef CAT
#undef CAT2
