"""CPU oracle for the hypervector encode / cosine top-k / propagate path.

Test infrastructure only: the product never imports this."""
