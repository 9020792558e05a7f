/* stub: empty (PNG output is off the compute path) */
