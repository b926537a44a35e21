	/* GB300 job_core: replaces the job_core() call of search() */
	if (!pa_context) pa_context = make_ctx(sett);
	{
	  pa_opts po = { opts->trl, opts->white_flag, opts->s0_flag,
	                 strcmp(opts->addsig, "") || strcmp(opts->range, "") };
	  pa_range pr;
	  int needed = 0;
	  memcpy(&pr, s_range, sizeof(pr));
	  status = pa_job_core(pa_context, pm, mm, nn, &po, &pr, &sgnlc, sgnlv, pa_sgnlv_cap,
	                       NULL, FNum, &needed);
	  if (status == PA_ERR_CAPACITY) {           /* nothing appended: grow sgnlv, run again */
	    pa_sgnlv_cap = needed;
	    sgnlv = (FLOAT_TYPE *)realloc(sgnlv, NPAR * (size_t)needed * sizeof(FLOAT_TYPE));
	    status = pa_job_core(pa_context, pm, mm, nn, &po, &pr, &sgnlc, sgnlv, pa_sgnlv_cap,
	                         NULL, FNum, &needed);
	  }
	  if (status != PA_OK) {
	    fprintf(stderr, "pa_job_core: %s\n", pa_last_error(pa_context));
	    exit(EXIT_FAILURE);
	  }
	}
