// mat_helpers.h -- the reference's host-side mat / vec helpers (matrix_vector_functions_intel_mkl.c,
// line numbers MVF:n below; the 64-bit and oneAPI variants have the same functions with their own
// index and element types).  Included once, inside extern "C", by api.cu, so that each of the three
// libraries gets them with its rsvd_int / rsvd_real.  Plain data movement and scalar loops in the
// reference's order; where the reference reads or writes past an object (a vector sized by the
// wrong dimension) only the entries inside both objects are touched.  Kept alike on purpose: the
// integer truncation in vector_get_min_element / vector_get_max_element (the reference compares
// the values converted to its index type, MVF:314-340).

// ---- printing (MVF:137-159)
void matrix_print(mat *M) {
    for (rsvd_int i = 0; i < M->nrows; i++) {
        for (rsvd_int j = 0; j < M->ncols; j++) std::printf("%f  ", (double)M->d[(size_t)j * M->nrows + i]);
        std::printf("\n");
    }
}
void vector_print(vec *v) {
    for (rsvd_int i = 0; i < v->nrows; i++) std::printf("%f\n", (double)v->d[i]);
}

// ---- element-wise (MVF:161-297)
void vector_set_data(vec *v, real *data) { std::memcpy(v->d, data, sizeof(real) * (size_t)v->nrows); }
void vector_scale(vec *v, real scalar) {
    for (rsvd_int i = 0; i < v->nrows; i++) v->d[i] = scalar * v->d[i];
}
void matrix_scale(mat *M, real scalar) {
    const size_t n = (size_t)M->nrows * (size_t)M->ncols;
    for (size_t i = 0; i < n; i++) M->d[i] = scalar * M->d[i];
}
void vector_copy(vec *d, vec *s) { std::memcpy(d->d, s->d, sizeof(real) * (size_t)s->nrows); }
void matrix_hard_threshold(mat *M, real TOL) {
    const size_t n = (size_t)M->nrows * (size_t)M->ncols;
    for (size_t i = 0; i < n; i++)
        if (std::fabs(M->d[i]) < TOL) M->d[i] = 0;
}
void vector_sub(vec *a, vec *b) {
    for (rsvd_int i = 0; i < a->nrows; i++) a->d[i] = a->d[i] - b->d[i];
}
void matrix_sub(mat *A, mat *B) {
    const size_t n = (size_t)A->nrows * (size_t)A->ncols;
    for (size_t i = 0; i < n; i++) A->d[i] = A->d[i] - B->d[i];
}
// A -= u v^T (MVF:287-297)
void matrix_sub_column_times_row_vector(mat *A, vec *u, vec *v) {
    for (rsvd_int j = 0; j < A->ncols; j++)
        for (rsvd_int i = 0; i < A->nrows; i++) A->d[(size_t)j * A->nrows + i] -= u->d[i] * v->d[j];
}

// ---- reductions in the reference's order (MVF:314-455)
void vector_get_min_element(vec *v, rsvd_int *minindex, real *minval) {
    *minindex = 0;
    *minval = v->d[0];
    for (rsvd_int i = 0; i < v->nrows; i++) {
        const rsvd_int val = (rsvd_int)v->d[i];
        if (val < *minval) {
            *minval = (real)val;
            *minindex = i;
        }
    }
}
void vector_get_max_element(vec *v, rsvd_int *maxindex, real *maxval) {
    *maxindex = 0;
    *maxval = v->d[0];
    for (rsvd_int i = 0; i < v->nrows; i++) {
        const rsvd_int val = (rsvd_int)v->d[i];
        if (val > *maxval) {
            *maxval = (real)val;
            *maxindex = i;
        }
    }
}
real vector_dot_product(vec *u, vec *v) {
    real acc = 0;
    for (rsvd_int i = 0; i < u->nrows; i++) acc += u->d[i] * v->d[i];
    return acc;
}
real get_matrix_max_abs_element(mat *M) {
    real mx = 0;
    const size_t n = (size_t)M->nrows * (size_t)M->ncols;
    for (size_t i = 0; i < n; i++)
        if (std::fabs(M->d[i]) > mx) mx = std::fabs(M->d[i]);
    return mx;
}
real get_matrix_column_norm_squared(mat *M, rsvd_int colnum) {
    real acc = 0;
    const real *c = M->d + (size_t)colnum * M->nrows;
    for (rsvd_int i = 0; i < M->nrows; i++) acc += c[i] * c[i];
    return acc;
}
real matrix_getmaxcolnorm(mat *M) {
    real mx = 0;
    for (rsvd_int j = 0; j < M->ncols; j++) {
        vec col{M->nrows, M->d + (size_t)j * M->nrows};
        const real nrm = vector_get2norm(&col);
        if (nrm > mx) mx = nrm;
    }
    return mx;
}
// column_norms(j) = ||M(:, j)||^2 (squared, as the reference stores them; MVF:445-455)
void compute_matrix_column_norms(mat *M, vec *column_norms) {
    for (rsvd_int j = 0; j < M->ncols; j++) column_norms->d[j] = get_matrix_column_norm_squared(M, j);
}
void invert_diagonal_matrix(mat *Dinv, mat *D) {
    for (rsvd_int i = 0; i < D->nrows; i++)
        Dinv->d[(size_t)i * Dinv->nrows + i] = (real)1.0 / D->d[(size_t)i * D->nrows + i];
}
// p = (v . u / ||u||^2) u (MVF:795-803)
void project_vector(vec *v, vec *u, vec *p) {
    const real dot = vector_dot_product(v, u);
    const real nrm = vector_get2norm(u);
    const real scale = dot / (nrm * nrm);
    for (rsvd_int i = 0; i < u->nrows; i++) p->d[i] = scale * u->d[i];
}

// Q = two passes of classical Gram-Schmidt over the columns of A, in the reference's order:
// column j minus its projections on columns 0..j-1 of the current Q, then normalised (MVF:817-844)
void build_orthonormal_basis_from_mat(mat *A, mat *Q) {
    const rsvd_int m = A->nrows, n = A->ncols;
    std::memcpy(Q->d, A->d, sizeof(real) * (size_t)m * (size_t)n);
    std::vector<real> pbuf((size_t)m);
    vec p{m, pbuf.data()};
    for (int pass = 0; pass < 2; pass++)
        for (rsvd_int j = 0; j < n; j++) {
            vec vj{m, Q->d + (size_t)j * m};
            for (rsvd_int i = 0; i < j; i++) {
                vec vi{m, Q->d + (size_t)i * m};
                project_vector(&vj, &vi, &p);
                vector_sub(&vj, &p);
            }
            const real nrm = vector_get2norm(&vj);
            vector_scale(&vj, (real)1.0 / nrm);
        }
}

// H(:, 0) = the Householder vector of x(ind1:ind2) scaled so that I - H H^T reflects it: x's entries
// in [ind1, ind2), ||x(ind1:ind2)|| taken off H(ind1, 0), then H scaled by sqrt(2) / ||H||_F
// (rank_revealing_algorithms_intel_mkl.c:982-1004; H's other entries are left as they are)
void get_householder_matrix(vec *x, rsvd_int ind1, rsvd_int ind2, mat *H) {
    double nrm = 0.0;
    for (rsvd_int i = ind1; i < ind2; i++) {
        H->d[i] = x->d[i];
        nrm += (double)x->d[i] * (double)x->d[i];
    }
    H->d[ind1] = H->d[ind1] - (real)std::sqrt(nrm);
    const double f = (double)get_matrix_frobenius_norm(H);
    if (f > 0) matrix_scale(H, (real)std::sqrt(2.0 / (f * f)));
}

// ---- rows and selections (MVF:608-790)
void matrix_get_row(mat *M, rsvd_int i, vec *row_vec) {
    for (rsvd_int j = 0; j < M->ncols; j++) row_vec->d[j] = M->d[(size_t)j * M->nrows + i];
}
void matrix_set_row(mat *M, rsvd_int i, vec *row_vec) {
    for (rsvd_int j = 0; j < M->ncols; j++) M->d[(size_t)j * M->nrows + i] = row_vec->d[j];
}
// column c of src (rows r0 ...) into column c' of dst, over the rows both have
static void copy_col(const mat *src, rsvd_int cs, mat *dst, rsvd_int cd) {
    std::memcpy(dst->d + (size_t)cd * dst->nrows, src->d + (size_t)cs * src->nrows,
                sizeof(real) * (size_t)std::min(src->nrows, dst->nrows));
}
static void copy_row(const mat *src, rsvd_int rs, mat *dst, rsvd_int rd) {
    const rsvd_int n = std::min(src->ncols, dst->ncols);
    for (rsvd_int j = 0; j < n; j++) dst->d[(size_t)j * dst->nrows + rd] = src->d[(size_t)j * src->nrows + rs];
}
void matrix_get_selected_columns(mat *M, rsvd_int *inds, mat *Mc) {
    for (rsvd_int i = 0; i < Mc->ncols; i++) copy_col(M, inds[i], Mc, i);
}
void matrix_set_selected_columns(mat *M, rsvd_int *inds, mat *Mc) {
    for (rsvd_int i = 0; i < Mc->ncols; i++) copy_col(Mc, i, M, inds[i]);
}
void matrix_get_selected_rows(mat *M, rsvd_int *inds, mat *Mr) {
    for (rsvd_int i = 0; i < Mr->nrows; i++) copy_row(M, inds[i], Mr, i);
}
void matrix_set_selected_rows(mat *M, rsvd_int *inds, mat *Mr) {
    for (rsvd_int i = 0; i < Mr->nrows; i++) copy_row(Mr, i, M, inds[i]);
}
// S(i, j) = M(i, j) for j >= i (MVF:757-771)
void matrix_copy_symmetric(mat *S, mat *M) {
    for (rsvd_int j = 0; j < M->ncols; j++)
        for (rsvd_int i = 0; i <= std::min(j, M->nrows - 1); i++)
            S->d[(size_t)j * S->nrows + i] = M->d[(size_t)j * M->nrows + i];
}
void matrix_keep_only_upper_triangular(mat *M) {
    for (rsvd_int j = 0; j < M->ncols; j++)
        for (rsvd_int i = j + 1; i < M->nrows; i++) M->d[(size_t)j * M->nrows + i] = 0;
}
// output(i) = input(inds(i)) for i < input->nrows (MVF:848-857)
void fill_vector_from_row_list(vec *input, vec *inds, vec *output) {
    for (rsvd_int i = 0; i < input->nrows; i++) output->d[i] = input->d[(rsvd_int)inds->d[i]];
}

// ---- leading / trailing blocks (MVF:859-1076)
void matrix_copy_first_rows(mat *M_out, mat *M) {
    for (rsvd_int i = 0; i < M_out->nrows; i++) copy_row(M, i, M_out, i);
}
void matrix_copy_first_columns(mat *M_out, mat *M) {
    for (rsvd_int j = 0; j < M_out->ncols; j++) copy_col(M, j, M_out, j);
}
void matrix_copy_first_columns_with_param(mat *D, mat *S, rsvd_int num_columns) {
    for (rsvd_int j = 0; j < num_columns; j++)
        for (rsvd_int i = 0; i < S->nrows; i++) D->d[(size_t)j * D->nrows + i] = S->d[(size_t)j * S->nrows + i];
}
void matrix_copy_first_k_rows_and_columns(mat *M_out, mat *M) {
    const rsvd_int k = M_out->ncols;
    for (rsvd_int j = 0; j < k; j++)
        for (rsvd_int i = 0; i < k; i++) M_out->d[(size_t)j * M_out->nrows + i] = M->d[(size_t)j * M->nrows + i];
}
// M_out = M(:, k+1:end)
void matrix_copy_all_rows_and_last_columns_from_indexk(mat *M_out, mat *M, rsvd_int k) {
    for (rsvd_int j = k; j < M->ncols; j++)
        for (rsvd_int i = 0; i < M->nrows; i++)
            M_out->d[(size_t)(j - k) * M_out->nrows + i] = M->d[(size_t)j * M->nrows + i];
}
void fill_matrix_from_first_rows(mat *M, rsvd_int k, mat *M_k) {
    for (rsvd_int i = 0; i < k; i++) copy_row(M, i, M_k, i);
}
void fill_matrix_from_last_rows(mat *M, rsvd_int k, mat *M_k) {
    for (rsvd_int i = 0; i < k; i++) copy_row(M, M->nrows - k + i, M_k, i);
}
void fill_matrix_from_first_columns(mat *M, rsvd_int k, mat *M_k) {
    for (rsvd_int j = 0; j < k; j++) copy_col(M, j, M_k, j);
}
void fill_matrix_from_last_columns(mat *M, rsvd_int k, mat *M_k) {
    for (rsvd_int j = 0; j < k; j++) copy_col(M, M->ncols - k + j, M_k, j);
}
// M_k = M(:, k:end) (0-based k)
void fill_matrix_from_last_columns_from_specified_one(mat *M, rsvd_int k, mat *M_k) {
    for (rsvd_int j = k; j < M->ncols; j++) copy_col(M, j, M_k, j - k);
}
// M_out = M(k:end, k:end) (0-based k)
void fill_matrix_from_lower_right_corner(mat *M, rsvd_int k, mat *M_out) {
    for (rsvd_int j = k; j < M->ncols; j++)
        for (rsvd_int i = k; i < M->nrows; i++)
            M_out->d[(size_t)(j - k) * M_out->nrows + (i - k)] = M->d[(size_t)j * M->nrows + i];
}
// M_k = M(:, I(1:k)), M(I(1:k), :), M(:, I(k+1:end)) (MVF:1012-1063)
void fill_matrix_from_first_columns_from_list(mat *M, vec *I, rsvd_int k, mat *M_k) {
    for (rsvd_int j = 0; j < k; j++) copy_col(M, (rsvd_int)I->d[j], M_k, j);
}
void fill_matrix_from_first_rows_from_list(mat *M, vec *I, rsvd_int k, mat *M_k) {
    for (rsvd_int i = 0; i < k; i++) copy_row(M, (rsvd_int)I->d[i], M_k, i);
}
void fill_matrix_from_last_columns_from_list(mat *M, vec *I, rsvd_int k, mat *M_k) {
    for (rsvd_int j = k; j < M->ncols; j++) copy_col(M, (rsvd_int)I->d[j], M_k, j - k);
}

// ---- resizes: *M is replaced by a new matrix (MVF:1078-1131)
static void resize_to(mat **M, mat *R) {
    matrix_delete(*M);
    *M = R;
}
void resize_matrix_by_columns(mat **M, rsvd_int k) {
    mat *R = matrix_new((*M)->nrows, k);
    fill_matrix_from_first_columns(*M, k, R);
    resize_to(M, R);
}
void resize_matrix_by_columns_from_end(mat **M, rsvd_int k) {
    mat *R = matrix_new((*M)->nrows, k);
    fill_matrix_from_last_columns(*M, k, R);
    resize_to(M, R);
}
void resize_matrix_by_rows(mat **M, rsvd_int k) {
    mat *R = matrix_new(k, (*M)->ncols);
    fill_matrix_from_first_rows(*M, k, R);
    resize_to(M, R);
}
void resize_matrix_by_rows_from_end(mat **M, rsvd_int k) {
    mat *R = matrix_new(k, (*M)->ncols);
    fill_matrix_from_last_rows(*M, k, R);
    resize_to(M, R);
}

// ---- concatenation and permutation inverse (MVF:1133-1201)
// C = [A, B]: A's entries, then B's, in column-major order
void append_matrices_horizontally(mat *A, mat *B, mat *C) {
    const size_t na = (size_t)A->nrows * (size_t)A->ncols, nb = (size_t)B->nrows * (size_t)B->ncols;
    std::memcpy(C->d, A->d, sizeof(real) * na);
    std::memcpy(C->d + na, B->d, sizeof(real) * nb);
}
// C = [A; B]
void append_matrices_vertically(mat *A, mat *B, mat *C) {
    for (rsvd_int j = 0; j < A->ncols; j++)
        for (rsvd_int i = 0; i < A->nrows; i++) C->d[(size_t)j * C->nrows + i] = A->d[(size_t)j * A->nrows + i];
    for (rsvd_int j = 0; j < B->ncols; j++)
        for (rsvd_int i = 0; i < B->nrows; i++)
            C->d[(size_t)j * C->nrows + A->nrows + i] = B->d[(size_t)j * B->nrows + i];
}
// Iinv(I(i)) = i
void vector_build_rewrapped(vec *Iinv, vec *I) {
    for (rsvd_int i = 0; i < I->nrows; i++) Iinv->d[(rsvd_int)I->d[i]] = (real)i;
}
